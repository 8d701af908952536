"""GPU parity: the sm_103a scan through the C ABI against the reference's
recorded outputs and the C oracle (bit-exact hit sets, identical tables)."""
import ctypes

import numpy as np
import pytest

from _golden import FINDER_CASES, Case, rows_equal
from _keys import oracle_keys, table_rows
from beguidedoff_gb300 import _native, build
from beguidedoff_gb300 import cuda_search as CS
from beguidedoff_gb300.finder import beguidedoff, prepare_n_masks
from beguidedoff_gb300.genome_converter import encode_chromosomes
from beguidedoff_gb300.types import GuideInput
from oracle import oracle as O

pytestmark = pytest.mark.gpu

IUPAC = O.IUPAC_MASK


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build.build()
    assert _native.device_count() >= 1


@pytest.mark.parametrize("mode,epilogue", [(0, "device"), (1, "device"), (2, "device"),
                                           (3, "device"), ("auto", "device"), (2, "host")])
@pytest.mark.parametrize("name", FINDER_CASES)
def test_finder_tables_match_reference(name, mode, epilogue):
    case = Case(name)
    meta = case.meta
    f = beguidedoff(None, max_mismatches=meta["max_mismatches"],
                    n_top_offtargets=meta["n_top_offtargets"],
                    results_per_guide=meta["results_per_guide"],
                    max_results_per_guide=meta["max_results_per_guide"],
                    genome_data=case.genome(), scan_mode=mode, epilogue=epilogue)
    try:
        for ri, run in enumerate(meta["runs"]):
            t = f.search(guides=case.guides(GuideInput), verbose=False, **run["kwargs"])
            ok, why = rows_equal(table_rows(t), case.expected_rows(ri))
            assert ok, f"{name} mode {mode} run {ri}: {why}"
    finally:
        f.close()


@pytest.mark.parametrize("name", FINDER_CASES)
def test_seam_matches_reference_raw_calls(name):
    case = Case(name)
    g = case.genome()
    fwd, rc = prepare_n_masks(g)
    for i in range(case.meta["raw_calls"]):
        c = case.raw_call(i)
        ne = int(c["n_encoded"])
        arr, nm = (g["genome_forward"], fwd) if ne == 0 else (g["genome_rc"], rc)
        if len(c["guide_encoded"]) > CS.MAX_GUIDES:
            continue
        res, ovf, cnt = CS.search_genome_cuda(
            arr, g["total_bp"], c["guide_encoded"], c["pam_masks"], c["pam_lens"],
            c["pam_3prime"], int(c["max_mismatches"]), return_overflow=True,
            results_per_guide=int(c["results_per_guide"]), n_mask_packed=nm, n_encoded=ne)
        for gi in range(len(c["guide_encoded"])):
            sel = c["hit_guide"] == gi
            exp = list(zip(c["hit_pos"][sel].tolist(), c["hit_mm"][sel].tolist()))
            assert res[gi] == exp, (name, i, gi)
            assert cnt[gi] == int(c["counts"][gi])


def test_seam_5prime_exotic_and_overflow_flags():
    case = Case("seam_5prime")
    d = case.d
    g = case.genome()
    fwd, rc = prepare_n_masks(g)
    for i in range(case.meta["raw_calls"]):
        c = case.raw_call(i)
        minus = str(c["strand"]) == "-"
        res, ovf, cnt = CS.search_genome_cuda(
            g["genome_rc"] if minus else g["genome_forward"], g["total_bp"], d["guide_encoded"],
            d["pam_masks"], d["pam_lens"], c["pam_3prime"], int(c["max_mismatches"]),
            return_overflow=True, results_per_guide=int(c["results_per_guide"]),
            n_mask_packed=rc if minus else fwd, n_encoded=int(c["n_encoded"]))
        for gi in range(len(d["guide_encoded"])):
            sel = c["hit_guide"] == gi
            assert res[gi] == list(zip(c["hit_pos"][sel].tolist(), c["hit_mm"][sel].tolist()))
            assert cnt[gi] == int(c["counts"][gi])
            assert ovf[gi] == bool(c["overflow"][gi])


def _random_genome(seed, lens, n_frac=0.02):
    rng = np.random.default_rng(seed)
    total = int(sum(lens))
    blocks, pos = [], 0
    while pos < total:
        pos += int(rng.integers(2_000, 60_000))
        ln = int(rng.integers(1, 3_000))
        if pos + ln >= total:
            break
        blocks.append((pos, pos + ln))
        pos += ln
    g = _native.synth_genome(seed, lens, blocks, thresholds=(76, 128, 180))
    return g, rng


def _plant(genome, rng, guide, pam, n_sites, max_sub):
    """Plant sites of `guide` + a concrete PAM on both strands in place."""
    comp = {"A": "T", "C": "G", "G": "C", "T": "A"}
    expand = {"A": "A", "C": "C", "G": "G", "T": "T", "R": "AG", "Y": "CT", "M": "AC",
              "K": "GT", "S": "CG", "W": "AT", "H": "ACT", "B": "CGT", "V": "ACG", "D": "AGT",
              "N": "ACGT"}
    fwd, rc = genome["genome_forward"], genome["genome_rc"]
    offs, lens = genome["chrom_offsets"], genome["chrom_lengths"]
    code = {"A": 0, "C": 1, "G": 2, "T": 3}
    for _ in range(n_sites):
        s = list(guide)
        for p in rng.choice(20, size=int(rng.integers(0, max_sub + 1)), replace=False):
            s[p] = rng.choice([b for b in "ACGT" if b != s[p]])
        site = "".join(s) + "".join(rng.choice(list(expand[c])) for c in pam)
        if rng.random() < 0.5:
            site = "".join(comp[b] for b in reversed(site))
        ci = int(rng.integers(0, len(lens)))
        at = int(offs[ci] + rng.integers(0, lens[ci] - len(site)))
        for k, b in enumerate(site):
            p = at + k
            v = code[b]
            fwd[p >> 4] = (fwd[p >> 4] & ~np.uint32(3 << ((p & 15) * 2))) | np.uint32(v << ((p & 15) * 2))
            q = int(offs[ci] + lens[ci] - 1 - (p - offs[ci]))
            rc[q >> 4] = (rc[q >> 4] & ~np.uint32(3 << ((q & 15) * 2))) | np.uint32((3 - v) << ((q & 15) * 2))
            nm = genome["n_mask"]
            nm[p >> 3] &= np.uint8(~(1 << (7 - (p & 7))) & 0xFF)


MIXED_PAMS = ["NGG", "NG", "NNGRRT", "NNNRRT", "NRN", "TTTV", "SGG", "NAG", "G", "NNNNNN"]


@pytest.mark.parametrize("seed", [11, 12])
def test_random_mixed_pam_keys_equal_oracle(seed):
    genome, rng = _random_genome(seed, [700_000, 33, 410_000, 1_234_567])
    seqs, pams = [], []
    for i in range(48):
        s = "".join(rng.choice(list("ACGT"), 20))
        pam = MIXED_PAMS[i % len(MIXED_PAMS)]
        _plant(genome, rng, s, pam, 6, 5)
        seqs.append(s)
        pams.append(pam)
    exp = oracle_keys(genome, seqs, pams, 5)
    assert exp.size > 100
    f = beguidedoff(None, max_mismatches=5, genome_data=genome)
    try:
        for mode in (0, 1, 2, 3):
            f.scan_mode = mode
            got = f._scan(seqs, pams)
            assert got.size == exp.size and np.array_equal(got, exp), mode
    finally:
        f.close()


def test_autotuned_scan_equals_oracle():
    """scan_mode='auto': the tuner times every candidate on the genome and the
    chosen form (with its tuning, including per-family launches) returns the
    oracle's keys."""
    genome, rng = _random_genome(77, [900_000, 650_000])
    seqs, pams = [], []
    for i in range(60):
        s = "".join(rng.choice(list("ACGT"), 20))
        pam = MIXED_PAMS[i % 5]
        _plant(genome, rng, s, pam, 5, 5)
        seqs.append(s)
        pams.append(pam)
    exp = oracle_keys(genome, seqs, pams, 5)
    f = beguidedoff(None, max_mismatches=5, genome_data=genome)
    try:
        assert f.scan_mode == "auto"
        got = f._scan(seqs, pams)
        assert np.array_equal(got, exp)
        ch = f.last_choice
        assert ch is not None and len(ch.times_ms) >= 5 and ch.mode in (1, 2, 3)
        plan = f._plan(seqs, pams)
        plan.set_tuning(0, 0, 0, 1)   # one launch per family
        assert np.array_equal(f._engine.scan(plan, f._strands, [0, 3], 5, 2), exp)
        plan.close()
    finally:
        f.close()


@pytest.mark.parametrize("k", [0, 1, 2, 3, 4, 5, 6, 7])
def test_indexed_modes_every_k_equal_oracle(k):
    """Segment index (mode 2) and segment masks (mode 3) at every segment
    layout they compile, against the oracle; mode 3 also at each tuning."""
    genome, rng = _random_genome(40 + k, [400_000, 260_001])
    seqs, pams = [], []
    for i in range(70):
        s = "".join(rng.choice(list("ACGT"), 20))
        pam = MIXED_PAMS[i % len(MIXED_PAMS)]
        _plant(genome, rng, s, pam, 3, min(k, 5))
        seqs.append(s)
        pams.append(pam)
    exp = oracle_keys(genome, seqs, pams, k)
    f = beguidedoff(None, max_mismatches=k, genome_data=genome)
    try:
        plan = f._plan(seqs, pams)
        tunings = [(0, 0, 0), (1024, 32, 0), (2048, 64, 2), (1024, 128, 1)]
        seed = [(0, 0, 0), (0, 0, 0, 1), (1024, 0, 0, 0, 4), (0, 0, 2, 1, 4), (1024, 0, 0, 0, 3),
                (0, 0, 0, 0, 0, 1), (1024, 0, 0, 1, 4, 1), (2048, 0, 0, 1, 3, 1),
                (0, 0, 0, 0, 0, 0, 2), (1024, 0, 0, 1, 4, 0, 2), (0, 0, 0, 0, 0, 0, 0, 1),
                (1024, 0, 0, 1, 4, 0, 0, 1), (0, 0, 0, 0, 1, 1), (1024, 0, 0, 1, 1, 1),
                (0, 0, 0, 0, 1, 0, 0, 1), (2048, 0, 0, 0, 1, 0, 2), (0, 0, 0, 0, 1, 1, 1),
                (1024, 0, 0, 1, 3, 1, 1), (0, 0, 0, 0, 2, 1), (1024, 0, 0, 1, 2, 0, 0, 1),
                # prefiltered form: 2,048 and 4,096 positions, all families in one
                # launch or one launch per family
                (0, 0, 0, 0, 0, 1, 0, 0, 1), (4096, 0, 0, 0, 0, 1, 0, 0, 1),
                (2048, 0, 0, 1, 0, 1, 0, 0, 1)]
        for mode, tune in [(2, t) for t in seed] + [(3, t) for t in tunings]:
            plan.set_tuning(*tune)
            got = f._engine.scan(plan, f._strands, [0, 3], k, mode)
            assert got.size == exp.size and np.array_equal(got, exp), (mode, tune)
        # one launch per family, each family with its own form and tuning
        plan.set_tuning(0, 0, 0, 1)
        fam = plan.families()
        assert fam.min() >= 0 and fam.max() == len(MIXED_PAMS) - 1
        forms = [dict(form=1), dict(tolerance=1, chunk_sites=1024), dict(min_blocks=4),
                 dict(tolerance=1, min_blocks=4), dict(chunk_sites=1024, inline_entries=2),
                 dict(tolerance=1, min_blocks=1), dict(min_blocks=1, range_walk=1),
                 dict(tolerance=1, inline_entries=1, chunk_sites=1024, min_blocks=1),
                 dict(tolerance=1, prefilter=1), dict(tolerance=1, prefilter=1, chunk_sites=4096)]
        for fi in range(fam.max() + 1):
            plan.set_family_tuning(fi, **forms[fi % len(forms)])
        got = f._engine.scan(plan, f._strands, [0, 3], k, 2)
        assert np.array_equal(got, exp), "per-family"
        plan.close()
    finally:
        f.close()


@pytest.mark.parametrize("k,chunk", [(4, 2048), (4, 4096), (2, 2048), (3, 4096)])
def test_prefilter_headline_shape_equals_oracle(k, chunk):
    """The prefiltered form on the headline's shape: 100 NGG guides, many
    planted sites per guide (survivor queues fill, flush mid-chunk and carry
    over between chunks), N blocks, a short chromosome and junction
    straddlers; keys equal the oracle's, and a graph replay equals the plain
    launch."""
    genome, rng = _random_genome(500 + k, [1_500_000, 61, 1_100_003, 400_000])
    seqs = ["".join(rng.choice(list("ACGT"), 20)) for _ in range(100)]
    for s in seqs:
        _plant(genome, rng, s, "NGG", 12, k)
    pams = ["NGG"] * len(seqs)
    exp = oracle_keys(genome, seqs, pams, k)
    assert exp.size > 500
    f = beguidedoff(None, max_mismatches=k, genome_data=genome)
    try:
        plan = f._plan(seqs, pams)
        plan.set_tuning(chunk, 0, 0, 0, 0, 1, 0, 0, 1)
        got = f._engine.scan(plan, f._strands, [0, 3], k, 2)
        assert got.size == exp.size and np.array_equal(got, exp)
        # the index is consulted only for survivors: far fewer pairs than
        # the index alone evaluates
        pf_pairs = f._engine.pairs_evaluated()
        plan.set_tuning(chunk if chunk == 2048 else 0, 0, 0, 0, 1, 1)
        assert np.array_equal(f._engine.scan(plan, f._strands, [0, 3], k, 2), exp)
        assert pf_pairs < f._engine.pairs_evaluated()
        plan.set_tuning(chunk, 0, 0, 0, 0, 1, 0, 0, 1)
        g = _native.Graph(f._engine, plan, f._strands, [0, 3], k, 2)
        try:
            for _ in range(2):
                g.replay()
                n, keys = f._engine.collect()
                assert n == exp.size and np.array_equal(keys, exp)
        finally:
            g.close()
        plan.close()
    finally:
        f.close()


def _write_base(genome, ci, p, v, n=False):
    """Base code v (A0 C1 G2 T3) at forward position p of chromosome ci, its
    complement at the mirrored reverse-complement position, and the N bit."""
    fwd, rc, nm = genome["genome_forward"], genome["genome_rc"], genome["n_mask"]
    off, ln = int(genome["chrom_offsets"][ci]), int(genome["chrom_lengths"][ci])
    fwd[p >> 4] = (fwd[p >> 4] & ~np.uint32(3 << ((p & 15) * 2))) | np.uint32(v << ((p & 15) * 2))
    q = off + ln - 1 - (p - off)
    rc[q >> 4] = (rc[q >> 4] & ~np.uint32(3 << ((q & 15) * 2))) | np.uint32((3 - v) << ((q & 15) * 2))
    bit = np.uint8(1 << (7 - (p & 7)))
    nm[p >> 3] = (nm[p >> 3] | bit) if n else (nm[p >> 3] & np.uint8(~bit & 0xFF))


@pytest.mark.parametrize("chunk", [2048, 4096])
def test_prefilter_n_at_chunk_boundaries_equal_oracle(chunk):
    """The prefiltered form learns whether a chunk or its halo holds an N
    from the strand's N summary (one bit per 1,024 positions) and reads the N
    words of its survivors from global memory.  Sites planted across
    1,024-position boundaries of either strand, with a single N inside the
    window at or just past the boundary, so that for a chunk boundary the N
    lies in the previous chunk's halo only (the guide's base there is the
    base an N is stored as, so only the N correction tells the hit's
    mismatches): keys equal the oracle's."""
    genome, rng = _random_genome(900 + chunk, [300_000, 200_003])
    code = {"A": 0, "C": 1, "G": 2, "T": 3}
    off0, ln0 = int(genome["chrom_offsets"][0]), int(genome["chrom_lengths"][0])
    seqs = []
    for b in range(1024, ln0 - 1024, 1024 * 7):
        for strand in (0, 1):
            j = int(rng.integers(0, 3))           # the N at boundary + j
            d = int(rng.integers(1, 20))          # window start = boundary + j - d
            guide = list("".join(rng.choice(list("ACGT"), 20)))
            # the guide's base at the N: A on the forward strand (N is stored
            # as A there), T on the reverse strand (N reads as T)
            guide[d] = "A" if strand == 0 else "T"
            guide = "".join(guide)
            seqs.append(guide)
            site = guide + "AGG"
            if strand == 0:
                start = off0 + b + j - d
                for k, c in enumerate(site):
                    _write_base(genome, 0, start + k, code[c])
                _write_base(genome, 0, off0 + b + j, 0, n=True)
            else:
                # reverse-strand position r maps to forward off0 + ln0 - 1 - r
                r0 = b + j - d
                for k, c in enumerate(site):
                    _write_base(genome, 0, off0 + ln0 - 1 - (r0 + k), 3 - code[c])
                _write_base(genome, 0, off0 + ln0 - 1 - (b + j), 0, n=True)
    pams = ["NGG"] * len(seqs)
    for k in (1, 4):
        exp = oracle_keys(genome, seqs, pams, k)
        f = beguidedoff(None, max_mismatches=k, genome_data=genome)
        try:
            plan = f._plan(seqs, pams)
            plan.set_tuning(chunk, 0, 0, 0, 0, 1, 0, 0, 1)
            got = f._engine.scan(plan, f._strands, [0, 3], k, 2)
            assert got.size == exp.size and np.array_equal(got, exp), k
            # every planted site is a hit whose N counts as a mismatch
            mm = (exp & 63).astype(np.int64)
            assert (mm >= 1).sum() >= len(seqs)
            plan.close()
        finally:
            f.close()


@pytest.mark.parametrize("tune", [(2048, 0, 0, 0, 0, 1, 0, 0, 1), (4096, 0, 0, 0, 0, 1, 0, 0, 1),
                                  (0, 0, 0, 0, 1, 1), (0, 0, 0, 0, 3, 0), None])
def test_overflow_rescans_only_dropped_granules(tune):
    """More hits than a fresh engine's buffer holds (1,048,576 keys): poly-A
    and poly-T runs hit at every position on one strand each.  After
    bgo_scan_complete the buffer holds exactly the oracle's keys; with the
    chunk-listed forms (segment index, prefiltered) the rescan covered only
    the granules whose keys were dropped (fewer pairs than a second full scan),
    and the other forms (tune None: the plain form) scan everything again."""
    rng = np.random.default_rng(404)
    bases = np.frombuffer(b"ACGT", dtype=np.uint8)
    c1 = bytearray(rng.choice(bases, 2_500_000).tobytes())
    c1[200_000:1_000_000] = b"A" * 800_000
    c2 = bytearray(rng.choice(bases, 1_000_003).tobytes())
    c2[300_000:700_000] = b"T" * 400_000
    genome = encode_chromosomes([("chrA", bytes(c1)), ("chrB", bytes(c2))])
    seqs, pams = ["A" * 20, "T" * 20, "ACGTACGTACGTACGTACGT"], ["NNN", "NRG", "NGG"]
    exp = oracle_keys(genome, seqs, pams, 2)
    assert exp.size > (1 << 20)
    f = beguidedoff(None, max_mismatches=2, genome_data=genome)
    try:
        eng = _native.Engine(0)
        plan = f._plan(seqs, pams, engine=eng)
        mode = 2 if tune is not None else 0
        if tune is not None:
            plan.set_tuning(*tune)
        # one scan without overflow for the pair count of a full scan
        big = _native.Engine(0)
        big.reserve(exp.size)
        plan2 = f._plan(seqs, pams, engine=big)
        if tune is not None:
            plan2.set_tuning(*tune)
        big.launch(plan2, f._strands, [0, 3], 2, mode)
        assert big.complete(plan2, f._strands, [0, 3], 2, mode) == exp.size
        full_pairs = big.pairs_evaluated()
        plan2.close()
        big.close()
        assert eng.info()["hit_capacity"] < exp.size
        eng.launch(plan, f._strands, [0, 3], 2, mode)
        first = eng.hit_count()
        assert first == exp.size
        n = eng.complete(plan, f._strands, [0, 3], 2, mode)
        assert n == exp.size
        got_n, keys = eng.collect()
        assert got_n == exp.size and np.array_equal(keys, exp)
        pairs = eng.pairs_evaluated()
        if tune is not None:
            assert full_pairs < pairs < 2 * full_pairs, (full_pairs, pairs)
        plan.close()
        eng.close()
    finally:
        f.close()


def test_index_forms_that_outgrow_shared_memory_equal_oracle():
    """Families large enough that the requested segment-index form (768-thread
    CTAs, 2,048-position chunks) does not fit in shared memory run in the next
    form that fits (1,024-position chunks, then 8 warps) or compare every guide;
    the keys stay the oracle's in one launch and in per-family launches."""
    genome, rng = _random_genome(91, [300_000, 120_001])
    seqs, pams = [], []
    # at K = 5 with tolerance 1 the requested 768-thread, 2,048-position form
    # fits none of these: NNGRRT steps down to 1,024-position chunks, NG to
    # 512 threads, NRN to 8 warps, and NGG fits no form
    for fam, n in (("NRN", 250), ("NG", 200), ("NGG", 1500), ("NNGRRT", 150)):
        for i in range(n):
            s = "".join(rng.choice(list("ACGT"), 20))
            if i % 50 == 0:
                _plant(genome, rng, s, fam, 3, 5)
            seqs.append(s)
            pams.append(fam)
    exp = oracle_keys(genome, seqs, pams, 5)
    assert exp.size > 100
    f = beguidedoff(None, max_mismatches=5, genome_data=genome)
    try:
        plan = f._plan(seqs, pams)
        for tune in [(0, 0, 0, 0, 1, 1), (0, 0, 0, 0, 1, 0, 0, 1), (0, 0, 0, 0, 1, 0, 2)]:
            plan.set_tuning(*tune)
            got = f._engine.scan(plan, f._strands, [0, 3], 5, 2)
            assert np.array_equal(got, exp), tune
        for fam_tune in [dict(tolerance=1, min_blocks=1), dict(min_blocks=1, range_walk=1),
                         dict(min_blocks=1, inline_entries=2), dict(tolerance=1),
                         dict(tolerance=1, min_blocks=2)]:
            plan.set_tuning(0, 0, 0, 1)
            for fi in range(plan.families().max() + 1):
                plan.set_family_tuning(fi, **fam_tune)
            got = f._engine.scan(plan, f._strands, [0, 3], 5, 2)
            assert np.array_equal(got, exp), fam_tune
        plan.close()
    finally:
        f.close()


@pytest.mark.parametrize("seed", [31, 32])
def test_device_epilogue_tables_equal_host_assembly(seed):
    """Device epilogue (exact score ranks, on-target exclusion, editable
    window, below-threshold counts, per-row top-N candidates) against the host
    assembly of the oracle's keys: identical tables, over input rows that share
    scan keys with different editors and windows, on-targets taken from real
    hits, tied scores, thresholds, return_all and several n_top values."""
    genome, rng = _random_genome(seed, [600_000, 47, 350_000, 900_001])
    seqs, pams = [], []
    for i in range(24):
        s = "".join(rng.choice(list("ACGT"), 20))
        pam = MIXED_PAMS[i % len(MIXED_PAMS)]
        _plant(genome, rng, s, pam, 12, 5)
        seqs.append(s)
        pams.append(pam)
    seqs.append(seqs[0])   # a repeated (seq, pam) with its own on-target
    pams.append(pams[0])
    host = beguidedoff.host_only(genome, 5)
    host._scan = lambda sq, pm: oracle_keys(genome, sq, pm, 5)
    probe = host.search(guides=[GuideInput(f"p{i}", s, p, "3prime", 1, 20, "ABE")
                                for i, (s, p) in enumerate(zip(seqs, pams))],
                        return_all=True, verbose=False)
    hits = table_rows(probe)
    guides = []
    editors = [("ABE", 4, 8), ("CBE", 3, 9), ("CGE", 1, 20), ("ABE", -3, 2), ("CBE", 18, 25)]
    for i, (s, p) in enumerate(zip(seqs, pams)):
        mine = [h for h in hits if h["guide_rna_sequence"] == s]
        for j, (ed, a, b) in enumerate(editors[: 1 + i % len(editors)]):
            ot = {}
            if mine and (i + j) % 2 == 0:
                h = mine[int(rng.integers(0, len(mine)))]
                ot = dict(on_target_chrom=h["ot_chromosome"], on_target_pos=h["ot_position"],
                          on_target_strand=h["ot_strand"])
            guides.append(GuideInput(f"g{i % 20}", s, p, "3prime", a, b, ed,
                                     base_editor=f"{ed}{j}", **ot))
    f = beguidedoff(None, max_mismatches=5, genome_data=genome)
    try:
        for n_top in (1, 3, 50):
            f.n_top_offtargets = host.n_top_offtargets = n_top
            for kw in ({}, {"return_all": True}, {"count_score_threshold": 2.0},
                       {"count_score_threshold": 20.0, "return_all": True},
                       {"count_score_threshold": float("nan")}):
                exp = table_rows(host.search(guides=guides, verbose=False, **kw))
                got = table_rows(f.search(guides=guides, verbose=False, **kw))
                ok, why = rows_equal(got, exp)
                assert ok, f"n_top {n_top} {kw}: {why}"
                assert len(exp) > 0
    finally:
        f.close()


def test_device_epilogue_ties_and_chromosome_order():
    """Tens of thousands of hits tied on score across chromosomes whose names
    sort differently from their order: the device's order keys (score rank,
    name rank, local position, strand) and radix select give the host
    assembly's exact top-N."""
    from beguidedoff_gb300.genome_converter import encode_chromosomes

    unit = "T" + "ACGTACGTACGTACGTACGT"[1:] + "AGG"
    rng = np.random.default_rng(3)
    chroms = []
    for name, reps in (("chr10", 9000), ("chr2", 7000), ("chrX", 5000), ("chr1", 8000)):
        body = list(unit * reps)
        for p in rng.choice(len(body), size=len(body) // 40, replace=False):
            body[p] = "ACGT"[int(rng.integers(0, 4))]
        chroms.append((name, "".join(body).encode()))
    g = encode_chromosomes(chroms)
    guide = "ACGTACGTACGTACGTACGT"
    host = beguidedoff.host_only(g, 4)
    host._scan = lambda sq, pm: oracle_keys(g, sq, pm, 4)
    guides = [GuideInput("a", guide, "NGG", "3prime", 4, 8, "ABE"),
              GuideInput("b", guide, "NGG", "3prime", 1, 20, "CBE", on_target_chrom="chr2",
                         on_target_pos=24, on_target_strand="+"),
              GuideInput("a", guide, "NGN", "3prime", 2, 6, "CGE")]
    f = beguidedoff(None, max_mismatches=4, genome_data=g, results_per_guide=10_000_000)
    host.results_per_guide = 10_000_000
    try:
        for n_top in (1, 3, 7, 200):
            f.n_top_offtargets = host.n_top_offtargets = n_top
            for kw in ({}, {"count_score_threshold": 3.0}, {"return_all": True}):
                exp = table_rows(host.search(guides=guides, verbose=False, **kw))
                got = table_rows(f.search(guides=guides, verbose=False, **kw))
                ok, why = rows_equal(got, exp)
                assert ok, f"n_top {n_top} {kw}: {why}"
    finally:
        f.close()


def test_five_prime_pams_every_form_equals_oracle():
    """5'-PAM rows (window after the PAM) mixed with 3' rows, through every
    scan form and the indexed forms' tunings, against the C oracle."""
    genome, rng = _random_genome(91, [500_000, 300_001])
    k = 4
    seqs, pams, p3 = [], [], []
    for i in range(40):
        seqs.append("".join(rng.choice(list("ACGT"), 20)))
        pams.append(["TTTV", "NGG", "TTN", "NNGRRT"][i % 4])
        p3.append(0 if i % 2 == 0 else 1)
    gv = np.array([O.encode_guide(s_) for s_ in seqs], dtype=np.uint64)
    pm = np.zeros((len(seqs), 6), dtype=np.uint8)
    for i, pam in enumerate(pams):
        for j, ch in enumerate(pam):
            pm[i, j] = IUPAC[ch]
    pl = np.array([len(p_) for p_ in pams], dtype=np.uint8)
    p3 = np.array(p3, dtype=np.uint8)
    fwd, rc = O.prepare_n_masks(genome)
    exp = []
    for slot, (arr, nm, ne) in enumerate(((genome["genome_forward"], fwd, 0),
                                          (genome["genome_rc"], rc, 3))):
        _, keys = O.scan_strand(arr, genome["total_bp"], nm, gv, pm, pl, p3, k, ne)
        g_, pos, mm = O.split_keys(keys)
        exp.append((g_.astype(np.uint64) << np.uint64(39)) | (np.uint64(slot) << np.uint64(38))
                   | (pos.astype(np.uint64) << np.uint64(6)) | mm.astype(np.uint64))
    exp = np.sort(np.concatenate(exp))
    assert exp.size > 0
    f = beguidedoff(None, max_mismatches=k, genome_data=genome)
    try:
        plan = _native.Plan(f._engine, gv, pm, pl, p3)
        forms = [(0, ()), (1, ()), (2, ()), (2, (0, 0, 0, 1)), (2, (0, 0, 0, 0, 0, 1)),
                 (2, (1024, 0, 0, 1, 4, 0, 2)), (2, (0, 0, 0, 0, 0, 0, 0, 1)), (3, (2048, 64)),
                 # the prefiltered form (window offset = PAM length for 5' rows)
                 (2, (0, 0, 0, 0, 0, 1, 0, 0, 1)), (2, (4096, 0, 0, 0, 0, 1, 0, 0, 1)),
                 (2, (2048, 0, 0, 1, 0, 1, 0, 0, 1))]
        for mode, tune in forms:
            plan.set_tuning(*tune)
            got = f._engine.scan(plan, f._strands, [0, 3], k, mode)
            assert np.array_equal(got, exp), (mode, tune)
        plan.close()
    finally:
        f.close()


def test_forward_only_genome_and_large_k():
    """A genome without genome_rc (one strand) through the device path, and
    max_mismatches 8-9 where the indexed forms fall back to every guide."""
    genome, rng = _random_genome(93, [300_000, 180_001])
    seqs = ["".join(rng.choice(list("ACGT"), 20)) for _ in range(6)]
    for s_ in seqs:
        _plant(genome, rng, s_, "NGG", 3, 4)
    fwd_only = {k_: v for k_, v in genome.items() if k_ != "genome_rc"}
    guides = [GuideInput(f"g{i}", s_, "NGG", "3prime", 4, 8, "ABE") for i, s_ in enumerate(seqs)]
    host = beguidedoff.host_only(fwd_only, 4)
    host._scan = lambda sq, pm: oracle_keys(fwd_only, sq, pm, 4)
    f = beguidedoff(None, max_mismatches=4, genome_data=fwd_only)
    try:
        for kw in ({}, {"return_all": True, "count_score_threshold": 3.0}):
            ok, why = rows_equal(table_rows(f.search(guides=guides, verbose=False, **kw)),
                                 table_rows(host.search(guides=guides, verbose=False, **kw)))
            assert ok, (kw, why)
    finally:
        f.close()
    f = beguidedoff(None, max_mismatches=8, genome_data=genome)
    try:
        for k in (8, 9):
            exp = oracle_keys(genome, seqs[:2], ["NGG"] * 2, k)
            plan = f._plan(seqs[:2], ["NGG"] * 2)
            for mode in (2, 3):
                assert np.array_equal(f._engine.scan(plan, f._strands, [0, 3], k, mode), exp)
            plan.close()
    finally:
        f.close()


def test_epilogue_row_chunks_equal_one_call(monkeypatch):
    """Input rows split over several bgo_epilogue_run calls give the records,
    counts and tables of one call."""
    genome, rng = _random_genome(95, [400_000, 250_001])
    seqs = ["".join(rng.choice(list("ACGT"), 20)) for _ in range(12)]
    for s_ in seqs:
        _plant(genome, rng, s_, "NGG", 6, 4)
    guides = [GuideInput(f"g{i % 5}", s_, "NGG", "3prime", 1 + i % 5, 12, "ABE" if i % 2 else "CBE")
              for i, s_ in enumerate(seqs)]
    f = beguidedoff(None, max_mismatches=4, genome_data=genome)
    try:
        one = table_rows(f.search(guides=guides, verbose=False, count_score_threshold=4.0))
        monkeypatch.setattr(_native.Engine, "EPILOGUE_ROWS_PER_CALL", 5)
        many = table_rows(f.search(guides=guides, verbose=False, count_score_threshold=4.0))
        ok, why = rows_equal(many, one)
        assert ok and len(one) > 0, why
    finally:
        f.close()


def test_graph_replay_equals_launch():
    """A captured scan (bgo_graph_create / bgo_graph_launch) returns the same
    keys as ordinary launches, on every replay, for the plain and indexed forms."""
    genome, rng = _random_genome(21, [900_000, 500_000])
    seqs, pams = [], []
    for i in range(30):
        s = "".join(rng.choice(list("ACGT"), 20))
        _plant(genome, rng, s, MIXED_PAMS[i % 5], 4, 4)
        seqs.append(s)
        pams.append(MIXED_PAMS[i % 5])
    f = beguidedoff(None, max_mismatches=5, genome_data=genome)
    try:
        exp = oracle_keys(genome, seqs, pams, 5)
        gv = np.array([O.encode_guide(s) for s in seqs], dtype=np.uint64)
        pm = np.zeros((len(seqs), 6), dtype=np.uint8)
        for i, pam in enumerate(pams):
            for j, ch in enumerate(pam):
                pm[i, j] = IUPAC[ch]
        pl = np.array([len(p) for p in pams], dtype=np.uint8)
        plan = _native.Plan(f._engine, gv, pm, pl, np.ones(len(seqs), dtype=np.uint8))
        for mode in (0, 2, 3):
            g = _native.Graph(f._engine, plan, f._strands, [0, 3], 5, mode)
            for _ in range(2):
                g.replay()
                n, keys = f._engine.collect()
                assert n == exp.size and np.array_equal(keys, exp), mode
            g.close()
        plan.close()
    finally:
        f.close()


def test_graph_recaptures_after_hit_buffer_grows():
    """A graph captured before bgo_engine_reserve moved the hit buffer must
    not write to the old buffer: the next replay captures again and returns
    the exact keys."""
    unit = "T" + "ACGTACGTACGTACGTACGT"[1:] + "AGG"
    from beguidedoff_gb300.genome_converter import encode_chromosomes

    g = encode_chromosomes([("chr1", (unit * 1_100_000 + "A" * 30).encode())])
    exp = oracle_keys(g, ["ACGTACGTACGTACGTACGT"], ["NGG"], 4)
    f = beguidedoff(None, max_mismatches=4, genome_data=g)
    try:
        cap0 = f._engine.info()["hit_capacity"]
        assert exp.size > cap0
        plan = f._plan(["ACGTACGTACGTACGTACGT"], ["NGG"])
        for mode in (3, 2, 1):
            gr = _native.Graph(f._engine, plan, f._strands, [0, 3], 4, mode)
            gr.replay()
            n, keys = f._engine.collect()
            if keys is None:
                f._engine.reserve(n)
            gr.replay()
            n, keys = f._engine.collect()
            assert keys is not None and np.array_equal(keys, exp), mode
            gr.close()
        plan.close()
    finally:
        f.close()


def test_graph_recaptures_after_plan_index_rebuild():
    """A launch of the same plan with another max_mismatches or tolerance
    rebuilds (and frees) the index a graph was captured with: the next replay
    prepares and captures again, and returns the graph's own keys."""
    genome, rng = _random_genome(58, [500_000, 210_000])
    seqs, pams = [], []
    for i in range(40):
        s = "".join(rng.choice(list("ACGT"), 20))
        pam = MIXED_PAMS[i % 5]
        _plant(genome, rng, s, pam, 4, 4)
        seqs.append(s)
        pams.append(pam)
    exp4 = oracle_keys(genome, seqs, pams, 4)
    exp2 = oracle_keys(genome, seqs, pams, 2)
    f = beguidedoff(None, max_mismatches=4, genome_data=genome)
    try:
        plan = f._plan(seqs, pams)
        for mode in (2, 3):
            gr = _native.Graph(f._engine, plan, f._strands, [0, 3], 4, mode)
            gr.replay()
            assert np.array_equal(f._engine.collect()[1], exp4), mode
            # a direct launch at K = 2 rebuilds the plan's index
            assert np.array_equal(f._engine.scan(plan, f._strands, [0, 3], 2, mode), exp2)
            gr.replay()
            assert np.array_equal(f._engine.collect()[1], exp4), mode
            if mode == 2:
                # a tolerance change rebuilds it too; the re-capture uses it
                plan.set_tuning(0, 0, 0, 0, 1, 1)
                assert np.array_equal(f._engine.scan(plan, f._strands, [0, 3], 4, 2), exp4)
                plan.set_tuning(0, 0, 0, 0, 0, 0)
                assert np.array_equal(f._engine.scan(plan, f._strands, [0, 3], 4, 2), exp4)
                gr.replay()
                assert np.array_equal(f._engine.collect()[1], exp4)
            gr.close()
        plan.close()
    finally:
        f.close()


def test_strand_upload_in_place_equals_fresh_strands():
    """bgo_genome_upload replaces a resident strand's contents without
    reallocating: scans afterwards see only the new genome."""
    g1, rng = _random_genome(61, [300_000, 200_001])
    g2, _ = _random_genome(62, [300_000, 200_001])
    seqs = ["".join(rng.choice(list("ACGT"), 20)) for _ in range(12)]
    for s_ in seqs:
        _plant(g2, rng, s_, "NGG", 4, 3)
    pams = ["NGG"] * len(seqs)
    f = beguidedoff(None, max_mismatches=4, genome_data=g1)
    try:
        before = f._scan(seqs, pams)
        assert np.array_equal(before, oracle_keys(g1, seqs, pams, 4))
        m_fwd, m_rc = prepare_n_masks(g2)
        for st, arr, m in zip(f._strands, (g2["genome_forward"], g2["genome_rc"]), (m_fwd, m_rc)):
            st.upload(arr, m)
        f._strand_arrays = [g2["genome_forward"], g2["genome_rc"]]
        got = f._scan(seqs, pams)
        assert np.array_equal(got, oracle_keys(g2, seqs, pams, 4))
    finally:
        f.close()


def test_large_genome_sampled_ranges_equal_oracle():
    """96 Mbp, 64 NGG guides: full GPU key set; the oracle re-scans four
    sampled 300 kbp ranges per strand and every planted site is found."""
    genome, rng = _random_genome(5, [40_000_000, 56_000_000], n_frac=0.05)
    seqs = ["".join(rng.choice(list("ACGT"), 20)) for _ in range(64)]
    for s in seqs[:16]:
        _plant(genome, rng, s, "NGG", 25, 3)
    f = beguidedoff(None, max_mismatches=4, genome_data=genome)
    try:
        got = f._scan(seqs, ["NGG"] * len(seqs))
    finally:
        f.close()
    row, slot, pos, mm = _native.split_keys(got)
    gv = np.array([O.encode_guide(s) for s in seqs], dtype=np.uint64)
    pm = np.tile(np.array([15, 4, 4, 0, 0, 0], dtype=np.uint8), (len(seqs), 1))
    pl = np.full(len(seqs), 3, dtype=np.uint8)
    p3 = np.ones(len(seqs), dtype=np.uint8)
    fwd, rc = O.prepare_n_masks(genome)
    tb = genome["total_bp"]
    for s_i, (arr, nm, ne) in enumerate(((genome["genome_forward"], fwd, 0),
                                         (genome["genome_rc"], rc, 3))):
        for a in rng.integers(0, tb - 400_000, 4).tolist():
            b = a + 300_000
            _, keys = O.scan_strand(arr, tb, nm, gv, pm, pl, p3, 4, ne, a, b)
            eg, ep, em = O.split_keys(keys)
            sel = (slot == s_i) & (pos >= a) & (pos < b)
            assert np.array_equal(row[sel], eg) and np.array_equal(pos[sel], ep)
            assert np.array_equal(mm[sel], em)
    assert int(((row < 16) & (mm <= 3)).sum()) >= 16 * 25


def test_capi_error_paths():
    L = _native.lib()
    h = ctypes.c_void_p()
    assert L.bgo_genome_create(None, 0, 0, None, 0, 0, None, ctypes.byref(h)) == _native.BGO_ERR_ARG
    arr = np.zeros(4, dtype=np.uint32)
    assert L.bgo_genome_create(arr.ctypes.data, 4, 1 << 33, None, 0, 0, None,
                               ctypes.byref(h)) == _native.BGO_ERR_ARG
    assert "total_bp" in _native.last_error()
    eng = _native.Engine(0)
    n = ctypes.c_int64()
    assert L.bgo_scan_collect(eng.handle, None, 0, ctypes.byref(n), None) == _native.BGO_ERR_STATE
    s = _native.Strand(np.arange(100, dtype=np.uint32), 1600)
    assert s.info()["total_bp"] == 1600 and not s.info()["has_n_mask"]
    plan = _native.Plan(eng, np.array([1, 2, 3], dtype=np.uint64),
                        np.array([[15, 4, 4, 0, 0, 0], [15, 4, 4, 0, 0, 0], [4, 0, 0, 0, 0, 0]],
                                 dtype=np.uint8), np.array([3, 3, 0], dtype=np.uint8),
                        np.ones(3, dtype=np.uint8))
    assert plan.info() == {"n_families": 1, "n_guides": 3}
    ne = np.array([5], dtype=np.int32)
    arrp = (ctypes.c_void_p * 1)(s.handle.value)
    assert L.bgo_scan_launch(eng.handle, plan.handle, arrp, ne.ctypes.data, 1, 4, 0,
                             None) == _native.BGO_ERR_ARG
    keys = eng.scan(plan, [s], [0], 20)   # max_mm 20: every NGG site, rows 0 and 1
    counts, exp = O.scan_strand(arr_words := np.arange(100, dtype=np.uint32), 1600, None,
                                plan.guides, plan.pam_masks, plan.pam_lens, plan.pam_3prime,
                                20, 0)
    assert keys.size == exp.size > 0 and counts[2] == 0
    assert np.array_equal(_native.split_keys(keys)[2], O.split_keys(exp)[1])
    plan.close()
    s.close()
    eng.close()


def test_hit_buffer_growth_keeps_exact_output():
    """More hits than the initial device buffer: the engine grows and re-runs."""
    unit = "T" + "ACGTACGTACGTACGTACGT"[1:] + "AGG"
    case_seq = unit * 1_100_000 + "A" * 30
    from beguidedoff_gb300.genome_converter import encode_chromosomes

    g = encode_chromosomes([("chr1", case_seq.encode())])
    f = beguidedoff(None, max_mismatches=4, genome_data=g)
    try:
        cap0 = f._engine.info()["hit_capacity"]
        got = f._scan(["ACGTACGTACGTACGTACGT"], ["NGG"])
        assert f._engine.info()["hit_capacity"] > cap0
    finally:
        f.close()
    exp = oracle_keys(g, ["ACGTACGTACGTACGTACGT"], ["NGG"], 4)
    assert exp.size > cap0 and np.array_equal(got, exp)
