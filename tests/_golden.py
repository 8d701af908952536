"""Loader for the golden fixtures in tests/golden/ (recorded from the reference).

Each fixture is an .npz written by tests/golden/make_golden.py; this module
turns it back into a genome dict (the reference's .npz keys), guide rows,
search parameters, expected output rows and raw kernel-seam calls.
"""
import json
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TABLE_COLS = [
    "guide_rna_sequence", "base_editor", "ot_rank", "ot_chromosome", "ot_position",
    "ot_strand", "ot_sequence", "ot_pam", "n_mismatches", "mismatch_positions",
    "score", "n_offtargets_below_threshold",
]
FINDER_CASES = ["planted_ngg", "mixed_pam", "n_gate", "n_gate_nomask", "overflow",
                "overflow_capped", "repeats", "many_guides", "sacas9_21nt"]


@dataclass(frozen=True)
class Guide:
    guide_id: str
    guide_seq: str
    pam: str
    pam_position: str
    edit_window_start: int
    edit_window_end: int
    editor_type: str
    on_target_chrom: Optional[str] = None
    on_target_pos: Optional[int] = None
    on_target_strand: Optional[str] = None
    base_editor: Optional[str] = None


class _Arrays(dict):
    """Decompressed fixture arrays with the NpzFile ``files`` attribute."""

    @property
    def files(self):
        return list(self.keys())


class Case:
    def __init__(self, name):
        self.name = name
        with np.load(os.path.join(GOLDEN_DIR, name + ".npz"), allow_pickle=False) as z:
            self.d = _Arrays({k: z[k] for k in z.files})
        self.meta = json.loads(str(self.d["meta_json"]))

    def genome(self):
        d = self.d
        g = {k: d[k] for k in ("genome_forward", "genome_rc", "chrom_offsets", "chrom_lengths")
             if k in d.files}
        g["chrom_names"] = d["chrom_names"]
        g["total_bp"] = int(d["total_bp"])
        if "n_mask" in d.files:
            g["n_mask"] = d["n_mask"]
        return g

    def guides(self, cls=Guide):
        d = self.d
        out = []
        for i in range(len(d["g_id"])):
            oc = str(d["g_ot_chrom"][i]) or None
            op = int(d["g_ot_pos"][i])
            os_ = str(d["g_ot_strand"][i]) or None
            be = str(d["g_base_editor"][i]) or None
            out.append(cls(str(d["g_id"][i]), str(d["g_seq"][i]), str(d["g_pam"][i]), "3prime",
                           int(d["g_ws"][i]), int(d["g_we"][i]), str(d["g_editor"][i]),
                           on_target_chrom=oc, on_target_pos=None if op < 0 else op,
                           on_target_strand=os_, base_editor=be))
        return out

    def expected_rows(self, run):
        d = self.d
        n = self.meta["runs"][run]["n_rows"]
        rows = []
        for i in range(n):
            r = {}
            for c in TABLE_COLS:
                v = d[f"r{run}_{c}"][i]
                r[c] = float(v) if c == "score" else (int(v) if v.dtype.kind == "i" else str(v))
            rows.append(r)
        return rows

    def raw_call(self, i):
        d = self.d
        pre = f"raw{i}_"
        return {k[len(pre):]: d[k] for k in d.files if k.startswith(pre)}


def rows_equal(got, exp):
    """Exact comparison of two row lists; returns (ok, first difference)."""
    if len(got) != len(exp):
        return False, f"row count {len(got)} != {len(exp)}"
    for i, (a, b) in enumerate(zip(got, exp)):
        for c in TABLE_COLS:
            va, vb = a[c], b[c]
            if c == "score":
                if not (float(va) == float(vb) or abs(float(va) - float(vb)) <= 1e-12 * abs(float(vb))):
                    return False, f"row {i} col {c}: {va!r} != {vb!r}"
            elif str(va) != str(vb):
                return False, f"row {i} col {c}: {va!r} != {vb!r}"
    return True, ""
