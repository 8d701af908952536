"""Guide TSV input and the output table (beguidedoff/io.py:15-180), pandas-free.

``load_guides_from_tsv`` accepts the reference's two layouts (explicit
columns, or ``guide_rna_sequence`` + ``base_editor`` resolved through
``base_editor_profiles.tsv``) and numbers rows ``row_0, row_1, ...``.  Fields
are read as text; an empty field counts as missing, as pandas' NaN does.
"""
from typing import List, Optional

import numpy as np

from .base_editing import get_edit_window_from_profile, read_profiles
from .table import COLUMNS, INT_COLUMNS, Table
from .types import GuideInput, OffTarget

_EDITING_TO_TYPE = {"ABE": "ABE", "CBE": "CBE"}


def _read_tsv(path):
    with open(path) as fh:
        lines = [ln.rstrip("\n").rstrip("\r") for ln in fh]
    lines = [ln for ln in lines if ln != ""]
    if not lines:
        raise ValueError(f"empty input file {path}")
    cols = lines[0].split("\t")
    rows = []
    for ln in lines[1:]:
        f = ln.split("\t")
        f += [""] * (len(cols) - len(f))
        rows.append(dict(zip(cols, f)))
    return cols, rows


def _opt(row, col):
    v = row.get(col)
    return None if v is None or v.strip() == "" else v.strip()


def _opt_int(row, col):
    v = _opt(row, col)
    return None if v is None else int(float(v))


def load_guides_from_tsv(input_file: str, presets_path: Optional[str] = None) -> List[GuideInput]:
    cols, rows = _read_tsv(input_file)
    guides = []
    if "guide_seq" in cols:
        for idx, row in enumerate(rows):
            be = row.get("base_editor")
            base_editor = None if be is None else (be if be.strip() else "nan")
            guides.append(GuideInput(
                guide_id=f"row_{idx}", guide_seq=row["guide_seq"].strip().upper(),
                pam=row["pam"].strip().upper(), pam_position="3prime",
                edit_window_start=int(row["edit_window_start"]),
                edit_window_end=int(row["edit_window_end"]),
                editor_type=row["editor_type"].strip().upper(),
                on_target_chrom=_opt(row, "chromosome"), on_target_pos=_opt_int(row, "position"),
                on_target_strand=_opt(row, "on_target_strand"), base_editor=base_editor or None))
    elif "guide_rna_sequence" in cols and "base_editor" in cols:
        if presets_path is None:
            raise ValueError("presets_path is required when using profile-based input "
                             "(guide_rna_sequence + base_editor columns)")
        profiles = {r["name"]: r for r in read_profiles(presets_path)}
        for idx, row in enumerate(rows):
            base_editor = row["base_editor"].strip()
            start, end, pam = get_edit_window_from_profile(base_editor, presets_path)
            editing = profiles[base_editor].get("editing", "")
            if editing not in _EDITING_TO_TYPE:
                raise ValueError(f"Base editor '{base_editor}' has unrecognised editing type "
                                 f"'{editing}'. Expected one of: {sorted(_EDITING_TO_TYPE)}")
            guides.append(GuideInput(
                guide_id=f"row_{idx}", guide_seq=row["guide_rna_sequence"].strip().upper(),
                pam=pam.upper(), pam_position="3prime", edit_window_start=start,
                edit_window_end=end, editor_type=_EDITING_TO_TYPE[editing],
                on_target_chrom=_opt(row, "chromosome"), on_target_pos=_opt_int(row, "position"),
                on_target_strand=_opt(row, "strand_used"), base_editor=base_editor))
    else:
        raise ValueError("Input file must contain either (guide_seq, pam, ...) or "
                         f"(guide_rna_sequence, base_editor) columns. Found: {cols}")
    return guides


def offtargets_to_table(offtargets: List[OffTarget], n_offtargets_below_threshold: int = 0) -> Table:
    cols = {c: [] for c in COLUMNS}
    for rank, ot in enumerate(offtargets, start=1):
        cols["guide_rna_sequence"].append(ot.guide_seq)
        cols["base_editor"].append(ot.base_editor)
        cols["ot_rank"].append(rank)
        cols["ot_chromosome"].append(ot.chromosome)
        cols["ot_position"].append(ot.position)
        cols["ot_strand"].append(ot.strand)
        cols["ot_sequence"].append(ot.offtarget_seq)
        cols["ot_pam"].append(ot.genomic_pam)
        cols["n_mismatches"].append(ot.n_mismatches)
        cols["mismatch_positions"].append(",".join(map(str, ot.mismatch_positions)))
        cols["score"].append(round(ot.score, 6))
        cols["n_offtargets_below_threshold"].append(n_offtargets_below_threshold)
    out = {}
    for c in COLUMNS:
        if c in INT_COLUMNS:
            out[c] = np.asarray(cols[c], dtype=np.int64)
        elif c == "score":
            out[c] = np.asarray(cols[c], dtype=np.float64)
        else:
            out[c] = np.asarray(cols[c], dtype=object)
    return Table(out, COLUMNS)


def offtargets_to_dataframe(offtargets: List[OffTarget], n_offtargets_below_threshold: int = 0):
    """pandas.DataFrame when pandas is importable, else a Table."""
    t = offtargets_to_table(offtargets, n_offtargets_below_threshold)
    try:
        return t.to_pandas()
    except ImportError:
        return t
