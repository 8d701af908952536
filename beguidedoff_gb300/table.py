"""Output table with the reference's columns (beguidedoff/io.py:155-180).

``search()`` returns a ``pandas.DataFrame`` when pandas is importable (what the
reference returns) and this column store otherwise.  ``Table`` offers the part
of the DataFrame interface the reference's callers use: ``len``, ``empty``,
``columns``, column access, ``iloc`` rows, ``to_csv`` and ``to_pandas``.
"""
from typing import Dict, List, Sequence

import numpy as np

COLUMNS = [
    "guide_rna_sequence", "base_editor", "ot_rank", "ot_chromosome", "ot_position",
    "ot_strand", "ot_sequence", "ot_pam", "n_mismatches", "mismatch_positions", "score",
    "n_offtargets_below_threshold",
]
INT_COLUMNS = {"ot_rank", "ot_position", "n_mismatches", "n_offtargets_below_threshold"}


class Row(dict):
    """One table row; ``row["col"]`` like a pandas Series."""


class _ILoc:
    def __init__(self, table):
        self._t = table

    def __getitem__(self, i):
        n = len(self._t)
        if i < 0:
            i += n
        if not 0 <= i < n:
            raise IndexError(i)
        return Row((c, _py(self._t._cols[c][i])) for c in self._t.columns)


def _py(v):
    return v.item() if isinstance(v, np.generic) else v


class Table:
    def __init__(self, columns: Dict[str, Sequence] = None, order: List[str] = None):
        columns = columns or {}
        self.columns = list(order or columns.keys())
        self._cols = {c: np.asarray(columns[c]) for c in self.columns}
        lens = {len(v) for v in self._cols.values()}
        if len(lens) > 1:
            raise ValueError("columns of unequal length")

    def __len__(self):
        return len(next(iter(self._cols.values()))) if self._cols else 0

    @property
    def empty(self):
        return len(self) == 0

    @property
    def iloc(self):
        return _ILoc(self)

    def __getitem__(self, col):
        return self._cols[col]

    def rows(self):
        return [self.iloc[i] for i in range(len(self))]

    def to_csv(self, path, sep="\t", index=False):
        with open(path, "w") as fh:
            if not self.columns:
                fh.write("\n")
                return
            fh.write(sep.join(self.columns) + "\n")
            for i in range(len(self)):
                vals = []
                for c in self.columns:
                    v = _py(self._cols[c][i])
                    vals.append(repr(v) if isinstance(v, float) else str(v))
                fh.write(sep.join(vals) + "\n")

    def to_pandas(self):
        import pandas as pd

        return pd.DataFrame({c: self._cols[c] for c in self.columns}, columns=self.columns)

    def __repr__(self):
        return f"Table({len(self)} rows x {len(self.columns)} columns)"


def concat(tables: List[Table]) -> Table:
    tables = [t for t in tables if t.columns]
    if not tables:
        return Table()
    cols = tables[0].columns
    return Table({c: np.concatenate([t._cols[c] for t in tables]) for c in cols}, cols)


_PANDAS = None


def pandas_available():
    """Whether pandas imports (probed once per process)."""
    global _PANDAS
    if _PANDAS is None:
        try:
            import pandas  # noqa: F401
        except ImportError:
            _PANDAS = False
        else:
            _PANDAS = True
    return _PANDAS
