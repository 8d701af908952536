"""Workload generators used by the benchmarks (device side): the repeat-family
genome of the hit-dense configuration."""
import numpy as np
import pytest

from beguidedoff_gb300 import _native, build

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build.build()
    assert _native.device_count() >= 1


def _decode(words, total):
    w = np.asarray(words, dtype=np.uint32)
    codes = (w[:, None] >> (2 * np.arange(16, dtype=np.uint32))[None, :]) & 3
    return codes.reshape(-1)[:total].astype(np.uint8)


def _find_all(codes, pattern):
    """Start positions of an exact match of `pattern` (base codes)."""
    n, m = codes.size, pattern.size
    hit = np.ones(n - m + 1, dtype=bool)
    for k in range(m):
        hit &= codes[k:n - m + 1 + k] == pattern[k]
    return np.nonzero(hit)[0]


@pytest.mark.parametrize("div", [0.0, 0.1])
def test_repeat_genome_copies_and_strands(div):
    lens = [1_200_000, 800_001]
    rep = {"n_families": 3, "family_len": 300, "n_copies": 120, "divergence": div, "seed": 5}
    g = _native.synth_genome(9, lens, [(10_000, 12_000)], thresholds=(76, 128, 180),
                             repeats=rep)
    plain = _native.synth_genome(9, lens, [(10_000, 12_000)], thresholds=(76, 128, 180))
    total = g["total_bp"]
    fwd, rc = _decode(g["genome_forward"], total), _decode(g["genome_rc"], total)
    # the reverse-complement array mirrors each chromosome
    for off, ln in zip(g["chrom_offsets"].tolist(), g["chrom_lengths"].tolist()):
        assert np.array_equal(rc[off:off + ln], 3 - fwd[off:off + ln][::-1])
    assert np.array_equal(g["n_mask"], plain["n_mask"])
    fams = [np.array(["ACGT".index(c) for c in s], dtype=np.uint8)
            for s in g["repeat_families"]]
    assert len(fams) == 3 and all(f.size == 300 for f in fams)
    region = total // 120
    base = _decode(plain["genome_forward"], total)
    changed = np.nonzero(fwd != base)[0]
    # every change lies in one copy per region (N block excepted: encoded A)
    assert np.unique(changed // region).size <= 120
    if div == 0.0:
        found = 0
        for f in fams:
            fw = _find_all(fwd, f[:40])
            rv = _find_all(fwd, (3 - f[::-1])[:40])
            found += fw.size + rv.size
            # copies sit one per region
            assert np.unique(np.concatenate([fw, rv]) // region).size == fw.size + rv.size
        assert found >= 118   # the copy overlapping the N block may be masked
    else:
        # substitution rate of the copies against their consensus
        sub = [_best_alignment(fwd[r * region:(r + 1) * region], fams) for r in range(120)]
        sub = [d for d in sub if d is not None]
        assert len(sub) >= 110
        assert 0.08 < sum(sub) / (300 * len(sub)) < 0.12


def _best_alignment(seg, fams):
    """Substitutions of the best-placed family copy inside `seg`: 8-mer anchors
    of each family and orientation vote for a placement."""
    best = None
    for f in fams:
        for cand in (f, 3 - f[::-1]):
            votes = {}
            for a in range(0, cand.size - 8, 8):
                for st in _find_all(seg, cand[a:a + 8]).tolist():
                    votes[st - a] = votes.get(st - a, 0) + 1
            if not votes:
                continue
            s0, v = max(votes.items(), key=lambda kv: kv[1])
            if v >= 4 and 0 <= s0 <= seg.size - cand.size:
                d = int((seg[s0:s0 + cand.size] != cand).sum())
                best = d if best is None else min(best, d)
    return best


def test_gpu_converter_matches_reference_golden(tmp_path):
    """bgo_encode_genome gives the reference convert()'s bytes (the golden
    recorded from the reference) for every include_rc / include_n_mask."""
    import os

    from _golden import GOLDEN_DIR
    from beguidedoff_gb300 import genome_converter as GC

    d = np.load(os.path.join(GOLDEN_DIR, "convert.npz"))
    fa = tmp_path / "g.fa"
    fa.write_text(str(d["fasta_text"]))
    for rc in (True, False):
        for nm in (True, False):
            out = tmp_path / f"o{rc}{nm}.npz"
            GC.convert(str(fa), str(out), include_rc=rc, include_n_mask=nm, verbose=False,
                       device=0)
            got = np.load(out)
            pre = f"rc{int(rc)}_nm{int(nm)}_"
            exp_keys = sorted(k[len(pre):] for k in d.files if k.startswith(pre))
            assert sorted(got.files) == exp_keys
            for k in exp_keys:
                assert np.array_equal(got[k], d[pre + k]), (rc, nm, k)


def test_gpu_encoder_equals_host_encoder_on_random_fasta():
    from beguidedoff_gb300 import genome_converter as GC

    rng = np.random.default_rng(12)
    alphabet = np.frombuffer(b"ACGTacgtNnRYKMSWBDHVx-", dtype=np.uint8)
    probs = np.array([0.2] * 4 + [0.02] * 4 + [0.05, 0.03] + [0.004] * 12)
    probs /= probs.sum()
    chroms = []
    for i, ln in enumerate([0, 1, 15, 16, 17, 1000, 33_333, 250_001]):
        seq = rng.choice(alphabet, size=ln, p=probs).astype(np.uint8)
        if ln > 500:
            seq[100:300] = ord("N")
        chroms.append((f"c{i}", seq.tobytes()))
    for rc in (True, False):
        for nm in (True, False):
            host = GC.encode_chromosomes(chroms, rc, nm)
            dev = GC.encode_chromosomes(chroms, rc, nm, device=0)
            assert sorted(host) == sorted(dev)
            for k in host:
                assert np.array_equal(np.asarray(host[k]), np.asarray(dev[k])), (rc, nm, k)
