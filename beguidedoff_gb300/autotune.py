"""Scan autotuner: picks the scan form and its launch parameters for a plan.

The reference launches one fixed kernel shape (256 threads per block over
200 Mbp chunks, beguidedoff/cuda_search.py:420-470).  Here the best form
depends on the plan: the segment index (scan mode 2) wins when each PAM family
holds few guides per bucket, comparing every guide (mode 1) wins at large
max_mismatches where K + 1 short segments filter little, and the segment
masks (mode 3) or per-family launches can win in between.  The tuner times
each candidate on a sample of the resident genome with CUDA events
(bgo_scan_time) and keeps the fastest.  Choices are cached by the plan's
signature: max_mismatches and, per PAM family, the guide count rounded up to
a power of two.

Candidate parameters: scan mode; tile length (positions per warp chunk,
``chunk_sites``); guides per mask group (``group_guides``, mode 3); one
launch per PAM family (``split_families``, mode 2); CTAs per SM the kernel is
compiled for (``min_blocks``: 3 or 4 CTAs of 256 threads with up to 80 or 64
registers, or one CTA whose warps share one copy of the index: 768 threads
(1) or 512 (2), mode 2); mismatches tolerated per key region (``tolerance``: 0 with K + 1
regions, or 1 with K / 2 + 1 regions and substitution-expanded buckets,
mode 2); the prefiltered form (``prefilter``: a lossless byte-table test per
PAM-passing position in front of the tolerance-1 index, which then stays in
global memory; all families in one persistent launch unless split).
"""
from dataclasses import dataclass, field
from typing import Dict, List, Sequence, Tuple

import numpy as np

from . import _native

# (name, mode, (chunk_sites, group_guides, ctas_per_sm, split_families, min_blocks,
#               tolerance, inline_entries))
CANDIDATES: Tuple[Tuple[str, int, Tuple[int, ...]], ...] = (
    ("all-guides", 1, (0, 0, 0, 0, 0, 0, 0)),
    ("segment-index", 2, (0, 0, 0, 0, 0, 0, 0)),
    ("segment-index/i2", 2, (0, 0, 0, 0, 0, 0, 2)),
    ("segment-index/walk", 2, (0, 0, 0, 0, 0, 0, 0, 1)),
    ("segment-index/1024/occ4", 2, (1024, 0, 0, 0, 4, 0, 0)),
    ("segment-index/per-family", 2, (0, 0, 0, 1, 0, 0, 0)),
    ("segment-index/t1", 2, (0, 0, 0, 0, 0, 1, 0)),
    ("segment-index/t1/1024", 2, (1024, 0, 0, 0, 0, 1, 0)),
    ("segment-index/t1/per-family", 2, (0, 0, 0, 1, 0, 1, 0)),
    ("segment-index/t1/per-family/1024", 2, (1024, 0, 0, 1, 0, 1, 0)),
    ("segment-index/t1/cta768", 2, (0, 0, 0, 0, 1, 1, 0)),
    ("segment-index/t1/1024/cta768", 2, (1024, 0, 0, 0, 1, 1, 0)),
    ("segment-index/t1/i1/1024/cta768", 2, (1024, 0, 0, 0, 1, 1, 1)),
    ("segment-index/walk/cta768", 2, (0, 0, 0, 0, 1, 0, 0, 1)),
    ("segment-index/walk/1024/cta768", 2, (1024, 0, 0, 0, 1, 0, 0, 1)),
    ("segment-masks/2048x128", 3, (2048, 128, 0, 0, 0, 0, 0)),
    ("prefilter", 2, (2048, 0, 0, 0, 0, 1, 0, 0, 1)),
    ("prefilter/4096", 2, (4096, 0, 0, 0, 0, 1, 0, 0, 1)),
    ("prefilter/per-family", 2, (2048, 0, 0, 1, 0, 1, 0, 0, 1)),
)
TUNING_FIELDS = ("chunk_sites", "group_guides", "ctas_per_sm", "split_families", "min_blocks",
                 "tolerance", "inline_entries", "range_walk", "prefilter")
# per PAM family, timed on a plan holding that family alone:
# (name, form (0 segment index, 1 every guide), chunk_sites, min_blocks, tolerance,
#  inline_entries, range_walk[, prefilter])
FAMILY_CANDIDATES = (
    ("prefilter", 0, 2048, 0, 1, 0, 0, 1),
    ("prefilter/4096", 0, 4096, 0, 1, 0, 0, 1),
    ("every-guide", 1, 0, 0, 0, 0, 0),
    ("index", 0, 0, 0, 0, 0, 0),
    ("index/walk", 0, 0, 0, 0, 0, 1),
    ("index/i2", 0, 0, 0, 0, 2, 0),
    ("index/1024/occ4", 0, 1024, 4, 0, 0, 0),
    ("index/t1", 0, 0, 0, 1, 0, 0),
    ("index/t1/1024", 0, 1024, 0, 1, 0, 0),
    ("index/t1/1024/occ4", 0, 1024, 4, 1, 0, 0),
    ("index/walk/cta768", 0, 0, 1, 0, 0, 1),
    ("index/t1/cta768", 0, 0, 1, 1, 0, 0),
    ("index/t1/1024/cta768", 0, 1024, 1, 1, 0, 0),
    ("index/t1/i1/cta768", 0, 0, 1, 1, 1, 0),
    ("index/t1/i1/1024/cta768", 0, 1024, 1, 1, 1, 0),
    ("index/t1/cta512", 0, 0, 2, 1, 0, 0),
    ("index/t1/1024/cta512", 0, 1024, 2, 1, 0, 0),
)
PER_FAMILY_TUNING = (0, 0, 0, 1, 0, 0, 0, 0, 0)
INDEXED_MAX_K = 7


@dataclass
class Choice:
    name: str
    mode: int
    tuning: Tuple[int, ...]
    times_ms: Dict[str, float] = field(default_factory=dict)
    sample_bp: int = 0
    # per-family choice (name "per-family"): PAM -> (name, form, chunk_sites,
    # min_blocks, tolerance, inline_entries, range_walk, ms alone, prefilter)
    family: Dict[str, tuple] = field(default_factory=dict)

    def as_dict(self):
        tuning = tuple(self.tuning) + (0,) * (len(TUNING_FIELDS) - len(self.tuning))
        return {"name": self.name, "mode": self.mode,
                "tuning": dict(zip(TUNING_FIELDS, tuning)),
                "times_ms": {k: round(v, 4) for k, v in self.times_ms.items()},
                "family": {p: {"form": c[0], "ms": round(c[7], 4)} for p, c in
                           self.family.items()},
                "sample_bp": self.sample_bp}

    def apply(self, plan, pams: Sequence[str]) -> None:
        plan.set_tuning(*self.tuning)
        if not self.family:
            return
        fam = plan.families()
        done = set()
        for row, f in enumerate(fam.tolist()):
            if f < 0 or f in done:
                continue
            done.add(f)
            c = self.family.get(pams[row].upper())
            if c is not None:
                plan.set_family_tuning(f, chunk_sites=c[2], min_blocks=c[3], tolerance=c[4],
                                       form=c[1], inline_entries=c[5], range_walk=c[6],
                                       prefilter=c[8] if len(c) > 8 else 0)


def signature(pams: Sequence[str], max_mismatches: int) -> tuple:
    """Cache key: K and, per PAM family, the guide count rounded up to a power
    of two."""
    counts: Dict[str, int] = {}
    for p in pams:
        counts[p.upper()] = counts.get(p.upper(), 0) + 1
    return (int(max_mismatches),) + tuple(
        sorted((p, 1 << max(0, int(c - 1).bit_length())) for p, c in counts.items()))


SIZE_CLASSES = (16, 64, 256, 1024)


def coarse_signature(n_guides: int, max_mismatches: int) -> tuple:
    """Cache key for plans that mix families freely (serving batches): K and
    a size class of the guide count (<= 16, <= 64, <= 256, <= 1024, more)."""
    cls = next((i for i, c in enumerate(SIZE_CLASSES) if n_guides <= c), len(SIZE_CLASSES))
    return (int(max_mismatches), cls)


def candidates_for(max_mismatches: int, n_families: int) -> List[Tuple[str, int, tuple]]:
    out = []
    for name, mode, tune in CANDIDATES:
        if mode in (2, 3) and max_mismatches > INDEXED_MAX_K:
            continue
        if tune[3] and n_families < 2:
            continue
        out.append((name, mode, tune))
    return out


class Autotuner:
    """Times the candidates on the first ``sample_bp`` positions of each
    strand (a prefix of the host arrays, uploaded once)."""

    def __init__(self, engine, strand_arrays, n_masks, total_bp: int, device: int = 0,
                 sample_bp: int = 200_000_000, reps: int = 2, coarse: bool = False):
        self.engine = engine
        self.coarse = coarse   # one choice per (max_mismatches, size class): serving
        self.reps = reps
        self.sample_bp = int(min(total_bp, sample_bp))
        self.device = device
        self._arrays = strand_arrays
        self._masks = n_masks
        self._strands = None
        self.cache: Dict[tuple, Choice] = {}

    def _sample(self):
        if self._strands is None:
            n = self.sample_bp
            words, nbytes = (n + 15) // 16, (n + 7) // 8
            self._strands = []
            for arr, m in zip(self._arrays, self._masks):
                mm = None if m is None else np.ascontiguousarray(
                    np.pad(np.asarray(m)[:nbytes], (0, 16)))
                self._strands.append(_native.Strand(np.ascontiguousarray(arr[:words]), n, mm,
                                                    self.device))
        return self._strands

    def choose(self, plan, pams: Sequence[str], max_mismatches: int, stream=None) -> Choice:
        """The fastest candidate for this plan (cached by signature); the
        plan's tuning is set to it."""
        sig = coarse_signature(len(pams), max_mismatches) if self.coarse else \
            signature(pams, max_mismatches)
        hit = self.cache.get(sig)
        if hit is None:
            strands = self._sample()
            ne = [0, 3][:len(strands)]
            n_fam = len({p.upper() for p in pams})
            times: Dict[str, float] = {}
            best = None
            for name, mode, tune in candidates_for(max_mismatches, n_fam):
                plan.set_tuning(*tune)
                ms = self.engine.scan_time(plan, strands, ne, max_mismatches, mode,
                                           self.reps, stream)
                times[name] = ms
                if best is None or ms < best[0]:
                    best = (ms, name, mode, tune)
            hit = Choice(best[1], best[2], best[3], times, self.sample_bp)
            if n_fam >= 2 and max_mismatches <= INDEXED_MAX_K and hasattr(plan, "guides"):
                total, fam = self._per_family(plan, pams, max_mismatches, stream)
                times["per-family"] = total
                if total < best[0]:
                    hit = Choice("per-family", 2, PER_FAMILY_TUNING, times, self.sample_bp, fam)
            self.cache[sig] = hit
        hit.apply(plan, pams)
        return hit

    def _per_family(self, plan, pams: Sequence[str], max_mismatches: int, stream=None):
        """Each family timed alone in every family candidate; returns the sum
        of the best times and the choice per family (keyed by PAM)."""
        strands = self._sample()
        ne = [0, 3][:len(strands)]
        fam = plan.families()
        total, out = 0.0, {}
        for f in sorted(set(fam.tolist()) - {-1}):
            rows = np.nonzero(fam == f)[0]
            sub = _native.Plan(self.engine, plan.guides[rows], plan.pam_masks[rows],
                               plan.pam_lens[rows], plan.pam_3prime[rows], stream)
            try:
                best = None
                for cand in FAMILY_CANDIDATES:
                    name, form, chunk, minb, tol, inl, walk = cand[:7]
                    pf = cand[7] if len(cand) > 7 else 0
                    sub.set_tuning(chunk, 0, 0, 0, minb, tol, inl, walk, pf)
                    ms = self.engine.scan_time(sub, strands, ne, max_mismatches,
                                               1 if form == 1 else 2, self.reps, stream)
                    if best is None or ms < best[7]:
                        best = (name, form, chunk, minb, tol, inl, walk, ms, pf)
            finally:
                sub.close()
            out[pams[int(rows[0])].upper()] = best
            total += best[7]
        return total, out

    def close(self):
        for s in self._strands or []:
            s.close()
        self._strands = None
