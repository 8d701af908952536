"""The allocation-free scan entry point, bgo_scan_noalloc, against the regular
scan (bgo_plan_create + bgo_scan_launch + bgo_scan_collect).

bgo_scan_noalloc exists for callers that cannot call cudaMalloc: programs
whose own allocator already owns the GPU's memory, and latency-critical loops
where an allocation would synchronise the device.  Its scratch is one static
device array shared by every call, so these tests call it several times in a
row with different guide sets and check that nothing from an earlier call
leaks into a later one.  The hit sets are integer data and must be identical.
This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from beguidedoff_gb300 import _native, build
from beguidedoff_gb300.encoding import encode_dna, encode_guide_64bit
from beguidedoff_gb300.pam import encode_pam_mask

pytestmark = pytest.mark.gpu


def _encode(seqs, ps):
    gv = np.array([encode_guide_64bit(encode_dna(s)) for s in seqs], dtype=np.uint64)
    pm = np.stack([encode_pam_mask(p) for p in ps]).astype(np.uint8)
    pl = np.array([len(p) for p in ps], dtype=np.uint8)
    return gv, pm, pl, np.ones(len(seqs), dtype=np.uint8)


def _rows(rng, n, pams):
    seqs = ["".join(rng.choice(list("ACGT"), 20)) for _ in range(n)]
    return _encode(seqs, [pams[i % len(pams)] for i in range(n)])


def _noalloc(strands, rows, max_mm, capacity, stream=None, keys=None):
    gv, pm, pl, p3 = rows
    handles = (ctypes.c_void_p * len(strands))(*[s.handle.value for s in strands])
    ne = np.array([0, 3][:len(strands)], dtype=np.int32)
    if keys is None:
        keys = np.zeros(capacity, dtype=np.uint64)
    n = ctypes.c_int64(-1)
    rc = _native.lib().bgo_scan_noalloc(handles, ne.ctypes.data, len(strands), gv.ctypes.data,
                                        pm.ctypes.data, pl.ctypes.data, p3.ctypes.data, gv.size,
                                        max_mm, keys.ctypes.data, capacity, ctypes.byref(n), stream)
    return rc, n.value, keys[:max(n.value, 0)]


@pytest.fixture(scope="module")
def setup():
    build.build()
    assert _native.device_count() >= 1
    lens = [1_500_000, 700_001]
    blocks = [(20_000, 23_000), (900_000, 900_500), (1_600_000, 1_650_000)]
    g = _native.synth_genome(99, lens, blocks, thresholds=(76, 128, 180))
    from beguidedoff_gb300.finder import prepare_n_masks

    fwd_nm, rc_nm = prepare_n_masks(g)
    strands = [_native.Strand(g["genome_forward"], g["total_bp"], fwd_nm),
               _native.Strand(g["genome_rc"], g["total_bp"], rc_nm)]
    strands[0].packed = g["genome_forward"]
    strands[0].genome = g
    eng = _native.Engine(0)
    yield strands, eng
    for s in strands:
        s.close()
    eng.close()


def _regular(eng, strands, rows, max_mm):
    plan = _native.Plan(eng, *rows)
    try:
        return eng.scan(plan, strands, [0, 3][:len(strands)], max_mm, mode=1)
    finally:
        plan.close()


def _genome_rows(strands_packed, rng, n, pams):
    """Guides copied from the genome itself, so every set has hits."""
    from beguidedoff_gb300.encoding import extract_windows

    starts = rng.integers(0, 2_000_000, n)
    bases = extract_windows(strands_packed, starts, 20)
    seqs = ["".join("ACGT"[b] for b in row) for row in bases]
    ps = [pams[i % len(pams)] for i in range(n)]
    gv = np.array([encode_guide_64bit(encode_dna(s)) for s in seqs], dtype=np.uint64)
    pm = np.stack([encode_pam_mask(p) for p in ps]).astype(np.uint8)
    pl = np.array([len(p) for p in ps], dtype=np.uint8)
    return gv, pm, pl, np.ones(n, dtype=np.uint8)


def test_noalloc_equals_regular_scan_on_consecutive_calls(setup):
    strands, eng = setup
    rng = np.random.default_rng(5)
    set_a = _rows(rng, 60, ["NGG", "NG", "NNGRRT", "NRN", "TTTV"])
    set_b = _genome_rows(strands[0].packed, rng, 17, ["NNN", "NAG"])
    exp_a = _regular(eng, strands, set_a, 5)
    exp_b = _regular(eng, strands, set_b, 3)
    assert exp_a.size > 0 and exp_b.size > 0
    for rows, mm, exp, ns in ((set_a, 5, exp_a, 2), (set_b, 3, exp_b, 2), (set_a, 5, exp_a, 2)):
        rc, n, keys = _noalloc(strands[:ns], rows, mm, exp.size + 10)
        assert rc == 0, _native.last_error()
        assert n == exp.size
        assert np.array_equal(keys, exp)
    # one strand only, after a two-strand call
    exp_f = _regular(eng, strands[:1], set_b, 3)
    rc, n, keys = _noalloc(strands[:1], set_b, 3, exp_f.size)
    assert rc == 0 and n == exp_f.size and np.array_equal(keys, exp_f)


def test_noalloc_limits_are_enforced(setup):
    strands, _ = setup
    rng = np.random.default_rng(6)
    too_many = _rows(rng, _native.NOALLOC_MAX_GUIDES + 1, ["NGG"])
    rc, n, _ = _noalloc(strands, too_many, 4, 16)
    assert rc == _native.BGO_ERR_ARG
    assert str(_native.NOALLOC_MAX_GUIDES) in _native.last_error()
    # a capacity too small for the hits: exact count reported, nothing copied
    rows = _rows(rng, 8, ["NRN"])
    rc, n, _ = _noalloc(strands, rows, 20, 0)
    assert rc == _native.BGO_ERR_OOM and n > _native.NOALLOC_MAX_HITS
    rc, n2, keys = _noalloc(strands, _rows(np.random.default_rng(5), 60,
                                           ["NGG", "NG", "NNGRRT", "NRN", "TTTV"]), 5, 10 ** 6)
    assert rc == 0 and n2 > 0 and np.all(np.diff(keys.astype(np.int64)) >= 0)


def test_noalloc_equals_oracle(setup):
    """The same keys as the CPU oracle's restatement of the reference kernel,
    with guides copied from the genome (every row has hits)."""
    from _keys import oracle_keys

    strands, _ = setup
    rng = np.random.default_rng(7)
    starts = rng.integers(0, 2_000_000, 12)
    from beguidedoff_gb300.encoding import extract_windows

    bases = extract_windows(strands[0].packed, starts, 20)
    seqs = ["".join("ACGT"[b] for b in row) for row in bases]
    pams = [["NGG", "NRN", "NNGRRT"][i % 3] for i in range(len(seqs))]
    exp = oracle_keys(strands[0].genome, seqs, pams, 3)
    assert exp.size > 0
    for _ in range(2):
        rc, n, keys = _noalloc(strands, _encode(seqs, pams), 3, exp.size)
        assert rc == 0, _native.last_error()
        assert n == exp.size and np.array_equal(keys, exp)


def test_noalloc_short_buffer_empty_call_pamless_rows_and_stream(setup):
    """A capacity below the hit count returns BGO_OK, the exact count and an
    untouched key buffer; a call with no guide rows after a call with hits
    reports 0 hits (the counters are cleared); rows whose PAM length is 0 never
    match, as in the regular path; a call on a created stream gives the same
    keys."""
    strands, eng = setup
    rng = np.random.default_rng(8)
    rows = _genome_rows(strands[0].packed, rng, 9, ["NNN"])
    exp = _regular(eng, strands, rows, 3)
    assert exp.size > 2
    sentinel = np.full(exp.size - 1, 7, dtype=np.uint64)
    rc, n, _ = _noalloc(strands, rows, 3, exp.size - 1, keys=sentinel)
    assert rc == 0 and n == exp.size and np.all(sentinel == 7)
    empty = tuple(a[:0] for a in rows)
    rc, n, _ = _noalloc(strands, empty, 3, 4)
    assert rc == 0 and n == 0
    gv, pm, pl, p3 = rows
    pl0 = pl.copy()
    pl0[::3] = 0
    mixed = (gv, pm, pl0, p3)
    exp0 = _regular(eng, strands, mixed, 3)
    rc, n, keys = _noalloc(strands, mixed, 3, max(exp0.size, 1))
    assert rc == 0 and n == exp0.size and np.array_equal(keys, exp0)
    s = _native.Stream(0)
    try:
        rc, n, keys = _noalloc(strands, rows, 3, exp.size, stream=s.handle)
        assert rc == 0 and n == exp.size and np.array_equal(keys, exp)
    finally:
        s.close()
