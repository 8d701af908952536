"""The plain CPU-runnable configuration at its stated size: 10 Mbp over 2
chromosomes, 1% N in runs of 100-5,000 bp, 10 random NGG guides x 20 planted
sites with 0-4 substitutions, ABE window 4-8, max_mismatches 4.

tests/golden/config1.npz holds the tables the reference's own finder.search
returned for it (recorded through tests/golden/make_golden.py) and the hashes
of the genome arrays the reference's converter wrote; the genome itself is
rebuilt here by tests/golden/config1.py from a version-stable PCG64 stream.
"""
import os
import sys

import numpy as np
import pytest

from _golden import Case, rows_equal
from _keys import oracle_keys, table_rows
from beguidedoff_gb300.finder import beguidedoff
from beguidedoff_gb300.genome_converter import encode_chromosomes
from beguidedoff_gb300.types import GuideInput

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import config1 as C1  # noqa: E402


@pytest.fixture(scope="module")
def case():
    c = Case("config1")
    chroms, guides, on = C1.generate()
    g = encode_chromosomes(chroms)
    return c, g


def test_generator_and_converter_equal_the_recorded_genome(case):
    """The rebuilt genome, encoded by this package's converter, has the hashes
    of the arrays the reference's converter wrote (the converter is pinned at
    10 Mbp too)."""
    c, g = case
    d = c.d
    assert C1.digest(g["genome_forward"]) == str(d["sha_forward"])
    assert C1.digest(g["genome_rc"]) == str(d["sha_rc"])
    assert C1.digest(g["n_mask"]) == str(d["sha_n_mask"])
    assert [str(x) for x in g["chrom_names"]] == [str(x) for x in d["chrom_names"]]
    assert np.array_equal(g["chrom_offsets"], d["chrom_offsets"])
    assert int(g["total_bp"]) == int(d["total_bp"])


def test_oracle_and_host_assembly_equal_reference_tables(case):
    """The C oracle's hits through the finder's host assembly give the
    reference's tables, row for row."""
    c, g = case
    meta = c.meta
    f = beguidedoff.host_only(g, meta["max_mismatches"], meta["n_top_offtargets"])
    f._scan = lambda seqs, pams: oracle_keys(g, seqs, pams, meta["max_mismatches"])
    for ri, run in enumerate(meta["runs"]):
        t = f.search(guides=c.guides(GuideInput), verbose=False, **run["kwargs"])
        ok, why = rows_equal(table_rows(t), c.expected_rows(ri))
        assert ok, f"run {ri}: {why}"
    assert meta["runs"][0]["n_rows"] >= 200


@pytest.mark.gpu
@pytest.mark.parametrize("mode,tuning,epilogue", [
    ("auto", None, "device"), (2, (2048, 0, 0, 0, 0, 1, 0, 0, 1), "device"),
    (2, (4096, 0, 0, 0, 0, 1, 0, 0, 1), "host"), (0, None, "device")])
def test_gpu_search_equals_reference_tables(case, mode, tuning, epilogue):
    """search() on the GPU (autotuned, prefiltered, plain) equals the
    reference's tables."""
    c, g = case
    meta = c.meta
    f = beguidedoff(None, max_mismatches=meta["max_mismatches"],
                    n_top_offtargets=meta["n_top_offtargets"], genome_data=g, scan_mode=mode,
                    scan_tuning=tuning, epilogue=epilogue)
    try:
        for ri, run in enumerate(meta["runs"]):
            t = f.search(guides=c.guides(GuideInput), verbose=False, **run["kwargs"])
            ok, why = rows_equal(table_rows(t), c.expected_rows(ri))
            assert ok, f"mode {mode} run {ri}: {why}"
    finally:
        f.close()
