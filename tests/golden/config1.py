"""Deterministic generator of the plain CPU-runnable configuration: 2
chromosomes totalling 10 Mbp of i.i.d. uniform ACGT, 1% of bases in N runs of
100-5,000 bp, 10 random 20-nt guides with PAM NGG, each planted at 20 sites
with 0-4 uniformly placed substitutions next to an NGG (strands 50/50).

Every random draw comes from the raw output of numpy's PCG64 bit generator
(``random_raw``), whose stream is fixed across numpy versions, so the test on
any machine rebuilds the same genome as the one recorded through the
reference; the fixture keeps only its hashes and the reference's tables.
"""
import hashlib

import numpy as np

SEED = 20261204
CHROMS = (("chr1", 6_000_000), ("chr2", 4_000_000))
N_GUIDES = 10
SITES_PER_GUIDE = 20
MAX_SUB = 4
N_FRAC = 0.01
N_RUN = (100, 5_000)
MAX_MISMATCHES = 4
_BASES = np.frombuffer(b"ACGT", dtype=np.uint8)
_COMP = bytes.maketrans(b"ACGT", b"TGCA")


class Raw:
    """Integers from PCG64's raw 64-bit words."""

    def __init__(self, seed):
        self.bg = np.random.PCG64(seed)

    def words(self, n):
        return np.asarray(self.bg.random_raw(int(n)), dtype=np.uint64)

    def below(self, k):
        return int(self.words(1)[0] % np.uint64(k))


def _bases(raw, n):
    w = raw.words((n + 31) // 32)
    codes = (w[:, None] >> (np.arange(32, dtype=np.uint64) * np.uint64(2))) & np.uint64(3)
    return _BASES[codes.ravel()[:n].astype(np.int64)].copy()


def _site(raw, guide):
    s = bytearray(guide.encode())
    n_sub = raw.below(MAX_SUB + 1)
    order = list(range(20))
    for i in range(19, 0, -1):   # Fisher-Yates on raw draws
        j = raw.below(i + 1)
        order[i], order[j] = order[j], order[i]
    for p in order[:n_sub]:
        others = [b for b in b"ACGT" if b != s[p]]
        s[p] = others[raw.below(3)]
    site = bytes(s) + bytes([_BASES[raw.below(4)]]) + b"GG"
    return site


def generate():
    """(chromosomes [(name, bytes)], guide sequences, on-targets
    {guide index: (chrom, 1-based position, strand)})."""
    raw = Raw(SEED)
    seqs = {}
    for name, n in CHROMS:
        s = _bases(raw, n)
        target, done = int(N_FRAC * n), 0
        while done < target:
            run = N_RUN[0] + raw.below(N_RUN[1] - N_RUN[0] + 1)
            at = raw.below(n - run)
            s[at:at + run] = ord("N")
            done += run
        seqs[name] = s
    guides = [_bases(raw, 20).tobytes().decode() for _ in range(N_GUIDES)]
    names = [c[0] for c in CHROMS]
    for g in guides:
        for _ in range(SITES_PER_GUIDE):
            site = _site(raw, g)
            minus = raw.below(2) == 1
            if minus:
                site = site.translate(_COMP)[::-1]
            c = names[raw.below(len(names))]
            at = raw.below(len(seqs[c]) - len(site))
            seqs[c][at:at + len(site)] = np.frombuffer(site, dtype=np.uint8)
    # one exact on-target per strand, excluded by coordinates
    on = {}
    site = (guides[0] + "TGG").encode()
    seqs["chr1"][1_000_000:1_000_023] = np.frombuffer(site, dtype=np.uint8)
    on[0] = ("chr1", 1_000_001, "+")
    site = (guides[1] + "AGG").encode().translate(_COMP)[::-1]
    seqs["chr2"][2_000_000:2_000_023] = np.frombuffer(site, dtype=np.uint8)
    on[1] = ("chr2", 2_000_023, "-")
    return [(n, seqs[n].tobytes()) for n in names], guides, on


def guide_inputs(GuideInput, guides, on):
    """The input rows: every guide with PAM NGG and the ABE window 4-8."""
    out = []
    for i, g in enumerate(guides):
        c, p, st = on.get(i, (None, None, None))
        out.append(GuideInput(f"row_{i}", g, "NGG", "3prime", 4, 8, "ABE",
                              on_target_chrom=c, on_target_pos=p, on_target_strand=st,
                              base_editor="ABE8e"))
    return out


def digest(arr):
    """sha256 of an array's bytes (the genome is checked by hash, not stored)."""
    return hashlib.sha256(np.ascontiguousarray(arr).tobytes()).hexdigest()
