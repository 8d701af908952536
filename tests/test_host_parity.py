"""Host post-processing of the finder against the reference's tables (CPU).

The device scan is replaced by the C oracle (hit keys in the device layout),
so this pins everything the finder does after the scan: dedup, strand
mapping, on-target exclusion, decode, CCTOP, editable window, truncation,
sort and top-N (beguidedoff/finder.py:119-679) against tests/golden.
"""
import logging

import pytest

from _golden import FINDER_CASES, Case, rows_equal
from _keys import oracle_keys, table_rows
from beguidedoff_gb300.finder import beguidedoff
from beguidedoff_gb300.types import GuideInput


@pytest.mark.parametrize("name", FINDER_CASES)
def test_host_assembly_matches_reference(name, caplog):
    case = Case(name)
    meta = case.meta
    genome = case.genome()
    f = beguidedoff.host_only(genome, meta["max_mismatches"], meta["n_top_offtargets"],
                              meta["results_per_guide"], meta["max_results_per_guide"])
    f._scan = lambda seqs, pams: oracle_keys(genome, seqs, pams, meta["max_mismatches"])
    for ri, run in enumerate(meta["runs"]):
        kw = run["kwargs"]
        caplog.clear()
        with caplog.at_level(logging.WARNING):
            t = f.search(guides=case.guides(GuideInput), verbose=False, **kw)
        ok, why = rows_equal(table_rows(t), case.expected_rows(ri))
        assert ok, f"{name} run {ri}: {why}"
        ref_warn = [w for w in run["warnings"] if "Truncated" in w]
        got_warn = [r.getMessage() for r in caplog.records if "Truncated" in r.getMessage()]
        assert len(ref_warn) == len(got_warn)
        for a, b in zip(ref_warn, got_warn):
            assert a.split(";")[0] == b.split(";")[0]


def test_errors_match_reference():
    case = Case("planted_ngg")
    f = beguidedoff.host_only(case.genome())
    f._scan = lambda seqs, pams: oracle_keys(case.genome(), seqs, pams, 4)
    g = case.guides(GuideInput)
    with pytest.raises(ValueError):
        f.search(verbose=False)
    with pytest.raises(ValueError):
        f.search(guides=[], verbose=False)
    bad = GuideInput("x", g[0].guide_seq, "NGG", "5prime", 4, 8, "CBE")
    with pytest.raises(ValueError):
        f.search(guides=[bad], verbose=False)
    nostrand = GuideInput("x", g[0].guide_seq, "NGG", "3prime", 4, 8, "CBE",
                          on_target_chrom="chr1", on_target_pos=10)
    with pytest.raises(ValueError):
        f.search(guides=[nostrand], verbose=False)
    unknown = GuideInput("x", g[0].guide_seq, "NGG", "3prime", 4, 8, "XBE")
    with pytest.raises(ValueError):
        f.search(guides=[unknown], return_all=True, verbose=False)


def test_empty_result_is_empty_table():
    case = Case("planted_ngg")
    f = beguidedoff.host_only(case.genome())
    f._scan = lambda seqs, pams: oracle_keys(case.genome(), seqs, pams, 0)
    t = f.search(guides=[GuideInput("x", "A" * 20, "TTTTTT", "3prime", 4, 8, "CBE")],
                 verbose=False)
    assert len(t) == 0 and t.empty
