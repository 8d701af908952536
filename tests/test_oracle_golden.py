"""The oracle against outputs recorded from the reference itself (CPU only).

Pins oracle/scan_oracle.c (the C restatement of search_chunk_kernel,
beguidedoff/cuda_search.py:163-314) on every raw kernel-seam call the
reference made, and oracle.oracle_search (the finder host logic,
beguidedoff/finder.py:119-679) on every recorded output table.  The NumPy
brute force cross-checks the C oracle on the same strands.
"""
import logging

import numpy as np
import pytest

from _golden import FINDER_CASES, Case, rows_equal
from oracle import oracle as O


def _strand_inputs(case, n_encoded):
    g = case.genome()
    fwd, rc = O.prepare_n_masks(g)
    if n_encoded == 0:
        return g["genome_forward"], fwd, g["total_bp"]
    return g["genome_rc"], rc, g["total_bp"]


@pytest.mark.parametrize("name", FINDER_CASES)
def test_raw_calls_match_reference(name):
    case = Case(name)
    for i in range(case.meta["raw_calls"]):
        c = case.raw_call(i)
        arr, nm, tbp = _strand_inputs(case, int(c["n_encoded"]))
        res, ovf, cnt = O.search_genome_seam(
            arr, tbp, c["guide_encoded"], c["pam_masks"], c["pam_lens"], c["pam_3prime"],
            int(c["max_mismatches"]), int(c["results_per_guide"]), nm, int(c["n_encoded"]))
        exp = {}
        for g, p, m in zip(c["hit_guide"].tolist(), c["hit_pos"].tolist(), c["hit_mm"].tolist()):
            exp.setdefault(g, []).append((p, m))
        for g in range(len(c["guide_encoded"])):
            assert res[g] == exp.get(g, []), (name, i, g)
            assert cnt[g] == int(c["counts"][g]), (name, i, g)


def test_seam_5prime_and_exotic_match_reference():
    case = Case("seam_5prime")
    d = case.d
    g = case.genome()
    fwd, rc = O.prepare_n_masks(g)
    for i in range(case.meta["raw_calls"]):
        c = case.raw_call(i)
        minus = str(c["strand"]) == "-"
        arr = g["genome_rc"] if minus else g["genome_forward"]
        res, ovf, cnt = O.search_genome_seam(
            arr, g["total_bp"], d["guide_encoded"], d["pam_masks"], d["pam_lens"],
            c["pam_3prime"], int(c["max_mismatches"]), int(c["results_per_guide"]),
            rc if minus else fwd, int(c["n_encoded"]))
        exp = {}
        for gi, p, m in zip(c["hit_guide"].tolist(), c["hit_pos"].tolist(), c["hit_mm"].tolist()):
            exp.setdefault(gi, []).append((p, m))
        for gi in range(len(d["guide_encoded"])):
            assert res[gi] == exp.get(gi, []), (i, gi)
            assert cnt[gi] == int(c["counts"][gi])
            assert ovf[gi] == bool(c["overflow"][gi])


@pytest.mark.parametrize("name", FINDER_CASES)
def test_oracle_tables_match_reference(name, caplog):
    case = Case(name)
    meta = case.meta
    cap = meta["max_results_per_guide"] or 2_621_440
    for ri, run in enumerate(meta["runs"]):
        kw = run["kwargs"]
        with caplog.at_level(logging.WARNING):
            rows = O.oracle_search(case.genome(), case.guides(), meta["max_mismatches"],
                                   meta["n_top_offtargets"], meta["results_per_guide"], cap,
                                   return_all=kw.get("return_all", False),
                                   count_score_threshold=kw.get("count_score_threshold"))
        ok, why = rows_equal(rows, case.expected_rows(ri))
        assert ok, f"{name} run {ri}: {why}"
        ref_trunc = any("Truncated" in w for w in run["warnings"])
        got_trunc = any("Truncated" in r.getMessage() for r in caplog.records)
        assert ref_trunc == got_trunc


@pytest.mark.parametrize("name", ["planted_ngg", "mixed_pam", "n_gate", "repeats"])
def test_c_oracle_matches_numpy_bruteforce(name):
    case = Case(name)
    g = case.genome()
    fwd, rc = O.prepare_n_masks(g)
    guides = case.guides()
    seqs = np.array([[{"A": 0, "C": 1, "G": 2, "T": 3}[c] for c in x.guide_seq] for x in guides],
                    dtype=np.uint8)
    gv = np.array([O.encode_guide(x.guide_seq) for x in guides], dtype=np.uint64)
    pm = np.zeros((len(guides), 6), dtype=np.uint8)
    for i, x in enumerate(guides):
        for j, ch in enumerate(x.pam):
            pm[i, j] = O.IUPAC_MASK[ch]
    pl = np.array([len(x.pam) for x in guides], dtype=np.uint8)
    p3 = np.ones(len(guides), dtype=np.uint8)
    mm = case.meta["max_mismatches"]
    for arr, nm, ne in ((g["genome_forward"], fwd, 0), (g["genome_rc"], rc, 3)):
        counts, keys = O.scan_strand(arr, g["total_bp"], nm, gv, pm, pl, p3, mm, ne)
        gi, pos, m = O.split_keys(keys)
        got = set(zip(gi.tolist(), pos.tolist(), m.tolist()))
        exp = O.bruteforce_strand(arr, g["total_bp"], nm, seqs, pm, mm, ne)
        assert got == exp
        assert int(counts.sum()) == len(exp)
