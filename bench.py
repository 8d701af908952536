"""Benchmark of the extensive off-target scan on one node.

Workload (default): the human-scale plain scan - a synthetic 3.1 Gbp genome of
24 chromosomes (47-249 Mbp, rescaled), GC 41% i.i.d., 5% N in blocks
(log-uniform 10 kb - 3 Mb), 100 random 20-nt guides with PAM NGG, ABE/CBE
windows 4-8 split 50/50, max_mismatches 4, both strands.  Seeded synthetic
data stands in for GRCh38 (not available offline).

A step = one scan of both strands against all guides.  ``value`` is guide-site
comparisons/s with the genome resident in HBM: guides x sum over strands of
(total_bp - 26) (the reference's per-strand site count) / kernel seconds,
timed with CUDA events on the launch stream.  ``e2e`` is the same metric
through the public finder API with every step uploading both strand arrays
and N masks from pinned host memory and reading the hits back.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--mode 0|1] [--genome-bp B] [--guides G]

Under torchrun each rank scans the full workload on its own GPU (weak
scaling, no data-path collective); value = all ranks' comparisons / the
slowest rank's time.  ``--impl reference`` times the CPU restatement of the
reference scan (oracle/) on all host cores on a bounded sample per step.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "guide-site comparisons/s"
UNIT = "cmp/s"
# DRAM bytes (read + write) of one prefiltered scan (the headline's autotuned
# form, 4,096-position chunks) of the plain workload at 300 Mbp, from ncu
# (profiles/scan_filter_kernel_ngg100_300mbp.md); traffic grows with the
# genome, so the line scales it to the run's length
NCU_TRAFFIC_PLAIN = (300_000_000, 150.274816e6 + 3.204352e6)
# the same capture's integer-pipe figures: the kernel is issue-bound, so these
# are its roofline in the integer-ALU sense
NCU_INT_PLAIN = {"issue_active_frac": 0.776, "alu_pipe_active_frac": 0.686,
                 "warps_active_frac": 0.438,
                 "source": "ncu smsp__issue_active, sm__pipe_alu_cycles_active, "
                           "sm__warps_active (pct of peak, active cycles) at 300 Mbp, "
                           "scan_filter_kernel<4, 4096, 1>"}


def make_workload(genome_bp, n_guides, seed=2):
    """Chromosome lengths, N blocks and guides of the human-scale config."""
    rng = np.random.default_rng(seed)
    n_chrom = 24
    raw = rng.uniform(47e6, 249e6, n_chrom)
    lens = np.floor(raw / raw.sum() * genome_bp).astype(np.int64)
    lens[0] += genome_bp - int(lens.sum())
    n_total = int(0.05 * genome_bp)
    blk = []
    while sum(blk) < n_total:
        blk.append(int(np.exp(rng.uniform(np.log(10_000), np.log(3_000_000)))))
    blk[-1] -= sum(blk) - n_total
    blk = [b for b in blk if b > 0]
    free = genome_bp - n_total
    gaps = np.floor(rng.dirichlet(np.ones(len(blk) + 1)) * free).astype(np.int64)
    order = rng.permutation(len(blk))
    blocks, pos = [], 0
    for i, bi in enumerate(order):
        pos += int(gaps[i])
        blocks.append((pos, pos + blk[bi]))
        pos += blk[bi]
    guides = ["".join(rng.choice(list("ACGT"), 20)) for _ in range(n_guides)]
    return lens, blocks, guides


_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x):
    """SplitMix64 finaliser (Steele, Lea and Flood 2014) on uint64 arrays,
    the generator of the device synthetic genome (bgo_synth_genome)."""
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def _cpu_bases(pos, seed, thresholds, total, repeats, fam_seq):
    """Base codes (0-3) of forward positions `pos` (int64), the device
    generator's pure function of (seed, position), without N."""
    u = pos.astype(np.uint64)
    lo, hi = int(pos.min()), int(pos.max()) + 1
    if hi - lo <= 2 * pos.size:
        # one hash per 8 positions over the covered range, read back as bytes
        w0 = lo >> 3
        ws = np.arange(w0, ((hi - 1) >> 3) + 1, dtype=np.uint64)
        with np.errstate(over="ignore"):
            h = _splitmix64(np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15) + ws)
        b8 = h.astype("<u8").view(np.uint8)[pos - 8 * w0]
    else:
        with np.errstate(over="ignore"):
            h = _splitmix64(np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15) + (u >> np.uint64(3)))
        b8 = ((h >> (np.uint64(8) * (u & np.uint64(7)))) & np.uint64(0xFF)).astype(np.uint8)
    t0, t1, t2 = (np.uint8(t) for t in thresholds)
    out = np.where(b8 < t0, 0, np.where(b8 < t1, 1, np.where(b8 < t2, 2, 3))).astype(np.uint8)
    if repeats:
        n_copies, flen = int(repeats["n_copies"]), int(repeats["family_len"])
        region = total // n_copies
        rseed = np.uint64(int(repeats.get("seed", seed)))
        div16 = np.uint64(int(round(float(repeats["divergence"]) * 65536)))
        r = pos // region
        with np.errstate(over="ignore"):
            hr = _splitmix64(rseed * np.uint64(0xD6E8FEB86659FD93) + r.astype(np.uint64))
        start = r * region + (hr % np.uint64(region - flen + 1)).astype(np.int64)
        i = pos - start
        inside = (r < n_copies) & (i >= 0) & (i < flen)
        if inside.any():
            ii, hh, pp = i[inside], hr[inside], u[inside]
            f = (((hh >> np.uint64(32)) & np.uint64(0xFFFFFF)) %
                 np.uint64(int(repeats["n_families"]))).astype(np.int64)
            rev = (hh >> np.uint64(63)) == 1
            fwd_b = fam_seq[f * flen + ii]
            rev_b = 3 - fam_seq[f * flen + flen - 1 - ii]
            b = np.where(rev, rev_b, fwd_b).astype(np.uint64)
            with np.errstate(over="ignore"):
                h2 = _splitmix64((rseed ^ np.uint64(0xA0761D6478BD642F)) + pp)
            sub = (h2 & np.uint64(0xFFFF)) < div16
            b = np.where(sub, (b + np.uint64(1) + (h2 >> np.uint64(16)) % np.uint64(3)) &
                         np.uint64(3), b)
            out[inside] = b.astype(np.uint8)
    return out


def cpu_repeat_families(repeats):
    """The repeat family sequences bgo_synth_genome_repeats inserts (strings)."""
    n = int(repeats["n_families"]) * int(repeats["family_len"])
    with np.errstate(over="ignore"):
        codes = (_splitmix64(np.uint64(int(repeats["seed"])) * np.uint64(0x9E3779B97F4A7C15) +
                             np.uint64(0x5851F42D4C957F2D) + np.arange(n, dtype=np.uint64))
                 >> np.uint64(62)).astype(np.int64)
    flen = int(repeats["family_len"])
    return ["".join("ACGT"[c] for c in codes[i:i + flen]) for i in range(0, n, flen)]


def cpu_synth_prefix(seed, lens, blocks, thresholds, n_pos, repeats=None):
    """The first n_pos positions of both strand arrays of the synthetic genome
    (bit-identical to bgo_synth_genome), built on the host with numpy: packed
    forward and reverse-complement words and their little-endian N masks, as
    the oracle scans them.  Only the reference arm uses it, so that the CPU
    baseline loads no product code."""
    lens = np.asarray(lens, dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]])
    total = int(lens.sum())
    n_pos = min(int(n_pos), total)
    bs = np.array([b[0] for b in blocks], dtype=np.int64)
    be = np.array([b[1] for b in blocks], dtype=np.int64)
    fam_seq = None
    if repeats:
        n = int(repeats["n_families"]) * int(repeats["family_len"])
        rseed = np.uint64(int(repeats.get("seed", seed)))
        with np.errstate(over="ignore"):
            fam_seq = (_splitmix64(rseed * np.uint64(0x9E3779B97F4A7C15) +
                                   np.uint64(0x5851F42D4C957F2D) + np.arange(n, dtype=np.uint64))
                       >> np.uint64(62)).astype(np.int64)

    def is_n(pos):
        k = np.searchsorted(be, pos, side="right")
        ok = k < bs.size
        res = np.zeros(pos.shape, dtype=bool)
        res[ok] = bs[k[ok]] <= pos[ok]
        return res

    n_words = (n_pos + 15) // 16
    fwd = np.zeros(n_words, dtype=np.uint32)
    rc = np.zeros(n_words, dtype=np.uint32)
    nm_f = np.zeros((n_pos + 7) // 8 + 16, dtype=np.uint8)
    nm_r = np.zeros_like(nm_f)
    step = 1 << 23
    for a in range(0, n_words * 16, step):
        q = np.arange(a, min(a + step, n_words * 16), dtype=np.int64)
        valid = q < total
        qf = np.minimum(q, total - 1)
        nf = is_n(qf) & valid
        bf = np.where(nf | ~valid, 0, _cpu_bases(qf, seed, thresholds, total, repeats, fam_seq))
        c = np.searchsorted(offs, qf, side="right") - 1
        src = offs[c] + lens[c] - 1 - (qf - offs[c])
        nr = is_n(src) & valid
        br = np.where(~valid, 0, 3 - np.where(nr, 0, _cpu_bases(src, seed, thresholds, total,
                                                                 repeats, fam_seq)))
        for arr, b in ((fwd, bf), (rc, br)):
            w = b.astype(np.uint32).reshape(-1, 16) << (2 * np.arange(16, dtype=np.uint32))
            arr[a // 16:a // 16 + w.shape[0]] = np.bitwise_or.reduce(w, axis=1)
        lim = min(q.size, n_pos - a)
        if lim > 0:
            for m, nb in ((nm_f, nf), (nm_r, nr)):
                bits = np.packbits(nb[:lim].astype(np.uint8), bitorder="little")
                m[a // 8:a // 8 + bits.size] |= bits
    return {"genome_forward": fwd, "genome_rc": rc, "total_bp": total, "n_pos": n_pos,
            "_nm_fwd_le": nm_f, "_nm_rc_le": nm_r}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def start(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self._proc = None
            return self
        threading.Thread(target=self._read, daemon=True).start()
        return self

    def _read(self):
        for line in self._proc.stdout:
            if self._stop.is_set():
                break
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        self._stop.set()
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
        return self.summary()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def dist_setup(backend=None):
    """Rank layout from the torchrun environment; for WORLD_SIZE > 1 a process
    group over NCCL (one GPU per rank), or the given backend (gloo in the CPU
    tests).  The scan shards as replicas: no collective on the data path."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist

        if backend is None:
            backend = "nccl"
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return ws, rank, local


def dist_max(x, ws):
    """Maximum of x over the ranks (the slowest rank's time)."""
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def replica_value(ws, units_per_rank, t_max_s):
    """Whole-job throughput of N replicas: all ranks' units over the slowest
    rank's time (weak scaling)."""
    return ws * units_per_rank / t_max_s


MIXED_FAMILIES = (("NGG", 0.40), ("NG", 0.20), ("NNGRRT", 0.15), ("NNNRRT", 0.15),
                  ("NRN", 0.10))
# hit-dense configuration: repeat families inserted into the genome
# (the configuration states 200,000 copies, which give 2.6e7 raw hits at
# max_mismatches 6; 1,000,000 give 4.5e7 and 2,500,000 8.0e7; the >1e8-hit
# regime it asks for takes 4,000,000 copies, one per 775 bp)
DENSE_REPEATS = {"n_families": 10, "family_len": 300, "n_copies": 4_000_000, "divergence": 0.10,
                 "seed": 17}
DENSE_EDITORS = (("ABE", 4, 8, "ABE8e"), ("CBE", 4, 8, "TadCBEd"), ("CGE", 5, 8, "CGBE"))
_IUPAC = {"A": "A", "C": "C", "G": "G", "T": "T", "R": "AG", "Y": "CT", "S": "CG", "W": "AT",
          "K": "GT", "M": "AC", "B": "CGT", "D": "AGT", "H": "ACT", "V": "ACG", "N": "ACGT"}


def guide_pams(args, n):
    """PAM of each guide: all NGG (plain configuration) or the mixed-family
    split of the batched and hit-dense configurations (restricted to
    ``--families`` when given: the same guides, only those families)."""
    if args.config == "plain":
        return ["NGG"] * n
    pams = []
    for pam, frac in MIXED_FAMILIES:
        pams += [pam] * int(round(frac * n))
    return (pams + ["NGG"] * n)[:n]


def select_families(args, guides, pams):
    keep = getattr(args, "families", None)
    if not keep:
        return guides, pams
    keep = {p.strip().upper() for p in keep.split(",")}
    idx = [i for i, p in enumerate(pams) if p in keep]
    return [guides[i] for i in idx], [pams[i] for i in idx]


SACAS9_FAMILIES = ("NNGRRT", "NNNRRT")


def sacas9_extend(guides, pams, seed=4):
    """SaCas9-family guides (NNGRRT, NNNRRT) are 21 nt: one more seeded base.
    The reference compares their first 20 bases and tests the PAM right after
    them (beguidedoff/encoding.py:70-75, cuda_search.py:239-275)."""
    rng = np.random.default_rng(seed)
    return [g + "ACGT"[int(rng.integers(0, 4))] if p in SACAS9_FAMILIES else g
            for g, p in zip(guides, pams)]


def sampled_ranges(lens, blocks, n_ranges, span, seed=5):
    """Position ranges [lo, hi) of a strand array for the parity check:
    chromosome junctions, N-block edges and seeded random starts (a quarter,
    a quarter, the rest)."""
    lens = np.asarray(lens, dtype=np.int64)
    total = int(lens.sum())
    rng = np.random.default_rng(seed)
    centres = list(np.cumsum(lens)[:-1][: max(1, n_ranges // 4)])
    edges = [b[0] for b in blocks][:: max(1, len(blocks) // max(1, n_ranges // 4))]
    centres += edges[: max(1, n_ranges // 4)]
    while len(centres) < n_ranges:
        centres.append(int(rng.integers(span, total - span)))
    out = []
    for c in sorted(int(x) for x in centres[:n_ranges]):
        lo = max(0, c - span // 2)
        hi = min(total - 26, lo + span)
        if out and lo < out[-1][1]:
            out[-1] = (out[-1][0], max(out[-1][1], hi))
        elif hi > lo:
            out.append((lo, hi))
    return out


def range_parity(genome_arrays, total, guides, pams, max_mm, gpu_keys, ranges, n_threads=0):
    """The GPU hit keys inside sampled ranges of both strands against the C
    oracle's rescan of those ranges (the oracle is the checker here, run in
    the CPU-baseline leg); keys row<<39 | strand<<38 | pos<<6 | mm."""
    from oracle import oracle as O

    gv = np.array([O.encode_guide(g[:20]) for g in guides], dtype=np.uint64)
    _, pm, pl, p3 = plan_arrays(guides, pams)
    gpu_keys = np.asarray(gpu_keys, dtype=np.uint64)
    g_slot = ((gpu_keys >> np.uint64(38)) & np.uint64(1)).astype(np.int64)
    g_pos = ((gpu_keys >> np.uint64(6)) & np.uint64(0xFFFFFFFF)).astype(np.int64)
    exp, got = [], []
    t0 = time.perf_counter()
    for slot, (arr, nm, ne) in enumerate(genome_arrays):
        for lo, hi in ranges:
            _, keys = O.scan_strand(arr, total, nm, gv, pm, pl, p3, max_mm, ne, lo, hi, n_threads)
            g, pos, mm = O.split_keys(keys)
            exp.append((g.astype(np.uint64) << np.uint64(39)) | (np.uint64(slot) << np.uint64(38))
                       | (pos.astype(np.uint64) << np.uint64(6)) | mm.astype(np.uint64))
            got.append(gpu_keys[(g_slot == slot) & (g_pos >= lo) & (g_pos < hi)])
    exp = np.sort(np.concatenate(exp)) if exp else np.zeros(0, dtype=np.uint64)
    got = np.sort(np.concatenate(got)) if got else np.zeros(0, dtype=np.uint64)
    return {"ranges": len(ranges) * len(genome_arrays),
            "bp": int(sum(hi - lo for lo, hi in ranges)) * len(genome_arrays),
            "keys_in_ranges": int(exp.size), "keys_equal": bool(np.array_equal(exp, got)),
            "oracle_s": round(time.perf_counter() - t0, 2),
            "ranges_detail": "chromosome junctions, N-block edges and seeded random starts, "
                             "both strands"}


def dense_guides(families, pams, seed=3):
    """Hit-dense guide set: 30% are 20-mers of a repeat consensus followed by a
    consensus PAM of the guide's family (where the consensus has one), the rest
    random."""
    rng = np.random.default_rng(seed)
    out = []
    for i, pam in enumerate(pams):
        if i % 10 < 3:
            fam = families[int(rng.integers(0, len(families)))]
            ok = [p for p in range(len(fam) - 20 - len(pam))
                  if all(fam[p + 20 + k] in _IUPAC[c] for k, c in enumerate(pam))]
            p = ok[int(rng.integers(0, len(ok)))] if ok else int(rng.integers(0, len(fam) - 26))
            out.append(fam[p:p + 20])
        else:
            out.append("".join(rng.choice(list("ACGT"), 20)))
    return out


def plan_arrays(guides, pams=None):
    from beguidedoff_gb300.encoding import encode_dna, encode_guide_64bit
    from beguidedoff_gb300.pam import encode_pam_mask

    n = len(guides)
    pams = pams or ["NGG"] * n
    gv = np.array([encode_guide_64bit(encode_dna(g)) for g in guides], dtype=np.uint64)
    pm = np.stack([encode_pam_mask(p) for p in pams]).astype(np.uint8)
    pl = np.array([len(p) for p in pams], dtype=np.uint8)
    return gv, pm, pl, np.ones(n, dtype=np.uint8)


def cpu_scan_rate(genome, guides, max_mm, target_s, n_threads=0, budget_bp=None, pams=None):
    """Oracle scan of both strands on a bounded prefix sample; returns
    (cmp/s, threads, sample description, seconds)."""
    from oracle import oracle as O

    gv, pm, pl, p3 = plan_arrays(guides, pams)
    fwd_nm, rc_nm = O.prepare_n_masks(genome) if budget_bp is None else (None, None)
    nms = (genome.get("_nm_fwd_le"), genome.get("_nm_rc_le"))
    if nms[0] is not None:
        fwd_nm, rc_nm = nms
    tb = genome["total_bp"]

    def run(span):
        t0 = time.perf_counter()
        for arr, nm, ne in ((genome["genome_forward"], fwd_nm, 0),
                            (genome["genome_rc"], rc_nm, 3)):
            O.scan_strand(arr, tb, nm, gv, pm, pl, p3, max_mm, ne, 0, span, n_threads)
        return time.perf_counter() - t0

    span = 2_000_000
    dt = run(span)
    span = int(min(tb - 26, max(span, span * target_s / max(dt, 1e-3))))
    dt = run(span)
    threads = n_threads or O.max_threads()
    rate = len(guides) * 2 * span / dt
    return rate, threads, f"positions [0, {span}) of both strands x {len(guides)} guides", dt


REFERENCE_SAMPLE_BP = 32_000_000
SHIM_RATE_FILE = os.path.join(ROOT, "tests", "golden", "reference_shim_rate.json")


def bench_reference(args, ws, rank):
    """The reference arm: the CPU restatement of the reference scan
    (oracle/scan_oracle.c, OpenMP on all host cores; the reference itself has
    no CPU implementation of this path and its kernel is Numba-JIT CUDA) on a
    bounded sample of the same workload: positions [0, REFERENCE_SAMPLE_BP) of
    both strands of the same synthetic genome, built on the host (no product
    code is loaded).  Each step is one timed scan of that sample."""
    if rank != 0:
        return
    from oracle import oracle as O

    lens, blocks, guides = make_workload(args.genome_bp, args.guides)
    pams = guide_pams(args, len(guides))
    reps = DENSE_REPEATS if args.config == "dense" else None
    span = int(min(REFERENCE_SAMPLE_BP, int(lens.sum()) - 26))
    t0 = time.perf_counter()
    g = cpu_synth_prefix(7, lens, blocks, (76, 128, 180), span + 64, repeats=reps)
    t_synth = time.perf_counter() - t0
    if args.config == "dense":
        guides = dense_guides(cpu_repeat_families(reps), pams)
    guides = sacas9_extend(guides, pams)
    guides, pams = select_families(args, guides, pams)
    args.guides = len(guides)
    gv = np.array([O.encode_guide(x[:20]) for x in guides], dtype=np.uint64)
    _, pm, pl, p3 = plan_arrays(guides, pams)
    tb = int(lens.sum())
    threads = O.max_threads()

    def step():
        t = time.perf_counter()
        for arr, nm, ne in ((g["genome_forward"], g["_nm_fwd_le"], 0),
                            (g["genome_rc"], g["_nm_rc_le"], 3)):
            O.scan_strand(arr, tb, nm, gv, pm, pl, p3, args.max_mm, ne, 0, span, 0)
        return time.perf_counter() - t

    for _ in range(args.warmup):
        step()
    times = [step() for _ in range(args.steps)]
    sec = statistics.median(times)
    value = len(guides) * 2 * span / sec
    sample = (f"positions [0, {span}) of both strands x {len(guides)} guides per step, "
              f"the same synthetic genome built on the host")
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic", "config": workload_config(args, lens),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample + " (oracle/scan_oracle.c, OpenMP)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "step_s": times, "synth_s": t_synth,
    }
    # the reference's own kernel body, run literally on one core through the
    # test-only CPU stand-ins (tests/golden/reference_shim_rate.py); it needs
    # the reference checkout, so it is measured in the build container and
    # read here
    try:
        shim = json.load(open(SHIM_RATE_FILE))
        out["cpu_baseline_reference_shim"] = dict(shim, kind="reference-shim")
    except (OSError, ValueError):
        pass
    print(json.dumps(out))


def workload_config(args, lens):
    if args.config == "dense":
        name = (f"hit-dense stress: synthetic {int(lens.sum()) / 1e9:.2f} Gbp, 24 chromosomes, "
                f"GC 41%, 5% N blocks, {DENSE_REPEATS['n_copies']} copies of "
                f"{DENSE_REPEATS['n_families']} random {DENSE_REPEATS['family_len']}-bp repeat "
                f"families at {DENSE_REPEATS['divergence']:.0%} divergence, {args.guides} guides "
                f"(30% from the repeat consensus, mixed PAM families as the batched config), "
                f"ABE/CBE/CGE windows, max_mismatches {args.max_mm}, both strands; a step = "
                f"scan + device epilogue (score ranks, window filter, below-threshold counts, "
                f"top-{3} candidates)")
        return {"workload": name, "genome_bp": int(lens.sum()), "guides": args.guides,
                "pam": "mixed", "max_mismatches": args.max_mm, "scan_mode": args.mode_requested,
                "repeats": DENSE_REPEATS,
                "l2": "inputs larger than L2 (bit planes of both strands ~2.3 GB)"}
    if args.config == "mixed":
        name = (f"batched mixed-PAM scan: synthetic {int(lens.sum()) / 1e9:.2f} Gbp, "
                f"24 chromosomes, GC 41%, 5% N blocks, {args.guides} random 20-nt guides "
                f"(NGG 40% NG 20% NNGRRT 15% NNNRRT 15% NRN 10%), "
                f"max_mismatches {args.max_mm}, both strands")
        pam = "mixed"
    else:
        name = (f"human-scale plain scan: synthetic {int(lens.sum()) / 1e9:.2f} Gbp, "
                f"24 chromosomes, GC 41%, 5% N blocks, {args.guides} random NGG guides, "
                f"max_mismatches {args.max_mm}, both strands")
        pam = "NGG"
    return {
        "workload": name,
        "genome_bp": int(lens.sum()), "guides": args.guides, "pam": pam,
        "max_mismatches": args.max_mm, "scan_mode": args.mode_requested,
        "l2": "inputs larger than L2 (bit planes of both strands ~2.3 GB)",
    }


def speedups(plain, batched_ms):
    """The batched form's speed-ups over the plain forms of plain_forms()."""
    out = {"speedup_vs_bruteforce": plain["brute_force"]["ms_per_step"] / batched_ms}
    if "per_family_same_kernel" in plain:
        out["speedup_vs_plain_same_kernel"] = (plain["per_family_same_kernel"]["ms_per_step"] /
                                               batched_ms)
    out["persistent_multi_family_vs_batched"] = (
        plain["persistent_multi_family"]["ms_per_step"] / batched_ms)
    return out


def plain_forms(f, plan, pams, args, sp, timed, comps, steps=3):
    """The same scan in the forms the batched one is compared with, each timed
    with CUDA events and its hit keys kept (sorted) for a key-set comparison:
    * brute_force: scan mode 0, one launch per PAM family and strand, every
      guide compared per PAM-passing position (the plain drop-in);
    * per_family_same_kernel: the autotuned index forms, one launch per PAM
      family, launched one after another without a graph;
    * persistent_multi_family: the prefiltered kernel over all families in one
      persistent launch (warps claim chunks family by family), graph-captured.
    The plan's autotuned tuning is restored afterwards."""
    from beguidedoff_gb300 import _native

    eng, st, K = f._engine, f._strands, args.max_mm
    choice = f.last_choice
    out = {}

    def run(name, mode, step_fn, n_steps):
        step_fn()
        eng.complete(plan, st, [0, 3], K, mode, sp)   # the buffer then fits every hit
        ms, tot = timed(step_fn, n_steps)
        n, k = eng.collect(sp)
        out[name] = {"mode": mode, "ms_per_step": tot / n_steps,
                     "value": comps / (tot / n_steps / 1e3), "hits_per_step": n, "_k": k}

    run("brute_force", 0, lambda: eng.launch(plan, st, [0, 3], K, 0, sp), max(1, steps - 1))
    if choice is not None:
        tune = tuple(choice.tuning) + (0,) * (9 - len(choice.tuning))
        if not tune[3]:   # a single-launch form: the same form, one launch per family
            plan.set_tuning(*(tune[:3] + (1,) + tune[4:]))
        run("per_family_same_kernel", 2, lambda: eng.launch(plan, st, [0, 3], K, 2, sp), steps)
        out["per_family_same_kernel"]["form"] = choice.name
    plan.set_tuning(2048, 0, 0, 0, 0, 1, 0, 0, 1)
    g = _native.Graph(eng, plan, st, [0, 3], K, 2)
    try:
        run("persistent_multi_family", 2, lambda: g.replay(sp), steps)
    finally:
        g.close()
    if choice is not None:
        choice.apply(plan, pams)
    return out


def bench_ours(args, ws, rank, local):
    import torch

    from beguidedoff_gb300 import _native, build
    from beguidedoff_gb300.finder import beguidedoff
    from beguidedoff_gb300.types import GuideInput

    build.build()
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    lens, blocks, guides = make_workload(args.genome_bp, args.guides)
    total = int(lens.sum())
    n_words, n_bytes = (total + 15) // 16, (total + 7) // 8
    pin = [_native.HostBuffer((n_words,), np.uint32), _native.HostBuffer((n_words,), np.uint32),
           _native.HostBuffer((n_bytes,), np.uint8)]
    dense = args.config == "dense"
    t0 = time.perf_counter()
    genome = _native.synth_genome(7, lens, blocks, thresholds=(76, 128, 180), device=local,
                                  out=[b.array for b in pin],
                                  repeats=DENSE_REPEATS if dense else None)
    t_synth = time.perf_counter() - t0
    pams = guide_pams(args, len(guides))
    if dense:
        guides = dense_guides(genome["repeat_families"], pams)
    guides = sacas9_extend(guides, pams)
    guides, pams = select_families(args, guides, pams)
    args.guides = len(guides)
    t0 = time.perf_counter()
    # a fixed mode runs every search() with the command line's launch tuning
    tuning = (args.chunk_sites, args.group_guides, args.ctas_per_sm, args.split_families,
              args.min_blocks, args.tolerance, args.inline_entries, args.range_walk,
              args.prefilter)
    f = beguidedoff(None, max_mismatches=args.max_mm, genome_data=genome,
                    device=f"cuda:{local}", scan_mode=args.mode,
                    scan_tuning=None if args.mode == "auto" else tuning)
    t_init = time.perf_counter() - t0
    nm_pin = []
    for m in (f._n_mask_fwd, f._n_mask_rc):
        hb = _native.HostBuffer((m.size,), np.uint8)
        hb.array[:] = m
        nm_pin.append(hb)
    gv, pm, pl, p3 = plan_arrays(guides, pams)
    plan = _native.Plan(f._engine, gv, pm, pl, p3)
    autotune = None
    if args.mode == "auto":
        t0 = time.perf_counter()
        f._mode_for(plan, pams)
        autotune = dict(f.last_choice.as_dict(), seconds=time.perf_counter() - t0)
        args.mode = f.last_choice.mode
    else:
        plan.set_tuning(*tuning)
    if dense:
        editors = [DENSE_EDITORS[i % 3] for i in range(len(guides))]
    else:
        editors = [("ABE", 4, 8, "ABE8e") if i % 2 == 0 else ("CBE", 4, 8, "TadCBEd")
                   for i in range(len(guides))]
    ginputs = [GuideInput(f"row_{i}", g, pams[i], "3prime", e[1], e[2], e[0], base_editor=e[3])
               for i, (g, e) in enumerate(zip(guides, editors))]
    eng = f._engine
    comps = args.guides * 2 * (total - 26)

    def timed(run_step, steps):
        """CUDA-event time of `steps` steps on the launch stream (ms list, total ms)."""
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        torch.cuda.synchronize()
        ev[0].record(stream)
        for k in range(steps):
            run_step()
            ev[k + 1].record(stream)
        torch.cuda.synchronize()
        return [ev[k].elapsed_time(ev[k + 1]) for k in range(steps)], ev[0].elapsed_time(ev[-1])

    # the plain forms for comparison: the brute-force kernel (one launch per
    # PAM family and strand, every guide compared) and the autotuned index
    # forms launched one per family without a graph
    plain = None
    if args.config == "mixed" and args.mode != 0:
        plain = plain_forms(f, plan, pams, args, sp, timed, comps)

    # -------- device-resident kernel timing (value) --------
    graph = None
    if args.mode in (2, 3) and not args.no_graph:
        graph = _native.Graph(eng, plan, f._strands, [0, 3], args.max_mm, args.mode)
        scan_step = lambda: graph.replay(sp)  # noqa: E731
    else:
        scan_step = lambda: eng.launch(plan, f._strands, [0, 3], args.max_mm, args.mode, sp)  # noqa: E731
    step = scan_step
    epi = None
    if dense:
        from beguidedoff_gb300.finder import epilogue_inputs
        from beguidedoff_gb300.scoring import score_ranks, threshold_rank

        inputs = epilogue_inputs([(i, g, (None, None, None)) for i, g in enumerate(ginputs)],
                                 threshold_rank(5.0), False)
        rank_table, _ = score_ranks()
        scan_step()
        eng.complete(plan, f._strands, [0, 3], args.max_mm, args.mode, sp)
        epi = {"records": 0}

        def step():
            scan_step()
            _, _, _, recs = eng.epilogue(plan, f._strands, inputs, f.chrom_offsets,
                                         f.chrom_lengths, f._chrom_rank, rank_table, 3, sp)
            epi["records"] = int(recs.size)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    n0 = eng.launch_count()
    clocks = ClockSampler(local).start()
    time.sleep(0.3)
    barrier(ws)
    step_ms, total_ms = timed(step, args.steps)
    barrier(ws)
    clk = clocks.stop()
    launches = eng.launch_count() - n0
    if dense:
        # the scan alone, to split the step between scan and epilogue
        scan_ms, scan_total = timed(scan_step, args.steps)
        epi.update({"scan_ms_per_step": scan_total / args.steps,
                    "epilogue_ms_per_step": (total_ms - scan_total) / args.steps,
                    "raw_hits_per_step": eng.hit_count(sp)})
    t_max = dist_max(total_ms / 1e3, ws)
    hits = eng.hit_count(sp)
    pairs = eng.pairs_evaluated(sp)
    # the timed form's hit keys, for the parity check and the plain forms
    gpu_keys = None
    if hits <= eng.info()["hit_capacity"]:
        _, gpu_keys = eng.collect(sp)
    if graph is not None:
        graph.close()
    if plain is not None:
        for form in plain.values():
            k = form.pop("_k", None)
            form["keys_equal"] = bool(gpu_keys is not None and k is not None and
                                      np.array_equal(k, gpu_keys))

    # -------- roofline: the compare loop is POPC-bound (1 POPC per pair) --------
    popc_peak = _native.probe_int_throughput(1, local)
    lop3_peak = _native.probe_int_throughput(0, local)
    per_launch_s = (total_ms / 1e3) / max(1, launches)
    pairs_per_launch = pairs / max(1, launches // args.steps) if args.mode == 0 else pairs
    achieved = pairs / (total_ms / 1e3 / args.steps) / 1e9
    # algorithmic bytes: the H, L and N planes of both strands, read once; the
    # prefiltered form in one launch streams H and L only, plus the strands'
    # N summaries (one bit per 1,024 positions; the N words that survivors of
    # chunks with an N read are data-dependent and not counted)
    tune_now = getattr(plan, "tuning", None) or {}
    words = (total + 31) // 32
    if tune_now.get("prefilter") and not tune_now.get("split_families"):
        plane_bytes = len(f._strands) * (2 * 4 * words + 4 * ((words + 1023) // 1024 + 1))
    else:
        plane_bytes = len(f._strands) * 3 * 4 * words
    hbm_peak = None
    try:
        hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, KeyError, ValueError):
        hbm_peak = 6800.0
    hbm_achieved = plane_bytes / (total_ms / 1e3 / args.steps) / 1e9

    # -------- end to end through the public API --------
    # (a) as the reference runs: the genome stays on the device between
    #     searches (beguidedoff/finder.py:321-377 caches it); each step is one
    #     search(): guides in, plan and epilogue inputs up, results down
    def search_step():
        return f.search(guides=ginputs, verbose=False, count_score_threshold=5.0)

    search_step()
    torch.cuda.synchronize()
    barrier(ws)
    n1 = eng.launch_count()
    x0 = eng.transfer()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        table = search_step()
    torch.cuda.synchronize()
    e2e_s = dist_max((time.perf_counter() - t0) / args.steps, ws)
    x1 = eng.transfer()
    e2e_launches = eng.launch_count() - n1
    h2d = (x1["h2d"] - x0["h2d"]) // args.steps
    d2h = (x1["d2h"] - x0["d2h"]) // args.steps
    e2e_split = {k: round(v, 5) for k, v in (f.last_batch or {}).items() if k.endswith("_s")}

    # (b) conservative: both strand arrays and N masks also uploaded from
    #     pinned host memory every step, into the same device buffers
    def upload_step():
        for st, arr, nm in zip(f._strands, pin[:2], nm_pin):
            st.upload(arr.array, nm.array, sp)
        return search_step()

    upload_step()
    torch.cuda.synchronize()
    x2 = eng.transfer()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        upload_step()
    torch.cuda.synchronize()
    e2e_up_s = dist_max((time.perf_counter() - t0) / args.steps, ws)
    x3 = eng.transfer()
    genome_bytes = (pin[0].array.nbytes + pin[1].array.nbytes + nm_pin[0].array.nbytes
                    + nm_pin[1].array.nbytes)
    e2e_up = {"value": ws * comps / e2e_up_s, "unit": UNIT, "s_per_step": e2e_up_s,
              "h2d_bytes_per_step": genome_bytes + (x3["h2d"] - x2["h2d"]) // args.steps,
              "d2h_bytes_per_step": (x3["d2h"] - x2["d2h"]) // args.steps}

    # -------- CPU baseline (oracle, all host cores, bounded sample) --------
    cpu, parity = None, None
    if rank == 0 and ws == 1 and not args.no_cpu:
        genome["_nm_fwd_le"], genome["_nm_rc_le"] = f._n_mask_fwd, f._n_mask_rc
        rate, threads, sample, dt = cpu_scan_rate(genome, guides, args.max_mm, args.cpu_seconds,
                                                  pams=pams)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": sample + f" ({dt:.1f} s, oracle/scan_oracle.c OpenMP)"}
        # the timed scan's keys inside sampled ranges against the oracle
        if gpu_keys is not None:
            n_r, span = (8, 1_000_000) if dense else (16, 2_000_000)
            parity = range_parity(
                [(genome["genome_forward"], f._n_mask_fwd, 0), (genome["genome_rc"], f._n_mask_rc, 3)],
                total, guides, pams, args.max_mm, gpu_keys,
                sampled_ranges(lens, blocks, n_r, span))

    # the batched mixed-PAM and serving records, on the resident genome
    subs = None
    if args.config == "plain" and ws == 1 and not args.no_subrecords:
        subs = {}
        t0 = time.perf_counter()
        subs["mixed1000"] = sub_mixed(f, lens, blocks, args, sp, timed)
        subs["mixed1000"]["seconds"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        subs["serve"] = serve_run(genome, total, local, 20.0, 6.0, 2, 16, 2048,
                                  baselines=("same_kernel",))
        subs["serve"]["seconds"] = time.perf_counter() - t0

    if rank == 0:
        value = replica_value(ws, comps, t_max / args.steps)
        popc = {"achieved_gops": achieved, "peak_gops": popc_peak, "frac": achieved / popc_peak,
                "compares_per_step": pairs, "lop3_peak_gops": lop3_peak,
                "peak_source": "measured live: bgo_probe_int_throughput"}
        if args.mode in (2, 3):
            # the segment index makes the compares sub-linear in guides: the
            # floor of a full scan is streaming both strands' planes once
            traffic, int_pipes = None, None
            if args.config == "plain" and not getattr(args, "families", ""):
                bp, nbytes = NCU_TRAFFIC_PLAIN
                traffic = nbytes * total / bp
                int_pipes = NCU_INT_PLAIN
            roof = {"bound": "hbm", "unit": "GB/s", "achieved": hbm_achieved, "peak": hbm_peak,
                    "frac": hbm_achieved / hbm_peak, "traffic": traffic,
                    "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum at "
                                      "300 Mbp, scaled by genome length" if traffic else None,
                    "bytes_per_step": plane_bytes,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
                    "int_popc": popc, "int_pipes_ncu": int_pipes,
                    # the brute-force formulation's integer roofline: 12 INT32 ops
                    # per guide-site comparison against the measured LOP3 rate; the
                    # index skips most comparisons, so the ratio exceeds 1
                    "bruteforce_equivalent": {
                        "ops_per_comparison": 12,
                        "achieved_tops": 12 * value / ws / 1e12,
                        "peak_tops": lop3_peak / 1e3,
                        "ratio": 12 * value / ws / 1e9 / lop3_peak}}
        else:
            roof = {"bound": "int", "unit": "Gop/s", "achieved": achieved, "peak": popc_peak,
                    "frac": achieved / popc_peak, "traffic": None,
                    "op": "POPC (one per PAM-passing position x guide pair)",
                    "peak_source": "measured live: bgo_probe_int_throughput(POPC)",
                    "pairs_per_step": pairs, "lop3_peak_gops": lop3_peak,
                    "hbm": {"achieved_gbs": hbm_achieved, "peak_gbs": hbm_peak,
                            "frac": hbm_achieved / hbm_peak, "bytes_per_step": plane_bytes}}
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic", "config": workload_config(args, lens),
            "roofline": roof,
            "cpu_baseline": cpu,
            "parity": parity,
            "subrecords": subs,
            "e2e": {"value": ws * comps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "s_per_step": e2e_s,
                    "rows": len(table), "launches": e2e_launches // args.steps,
                    "genome": "resident between searches, as the reference keeps it"},
            "e2e_genome_upload": e2e_up,
            "e2e_split_s": e2e_split,
            "gpu_launches": launches,
            "tuning": getattr(plan, "tuning", None),
            "autotune": autotune,
            "epilogue": epi,
            "graph": graph is not None,
            "plain_forms": plain,
            **(speedups(plain, 1e3 * t_max / args.steps) if plain else {}),
            "clocks": clk,
            "hits_per_step": hits,
            "step_ms": step_ms,
            "setup_s": {"synth": t_synth, "finder_init": t_init},
        }
        print(json.dumps(out))
    plan.close()
    f.close()
    for b in pin + nm_pin:
        b.close()


def serve_trace(rate, duration, seed=11):
    """Seeded request trace of the serving config: Poisson arrivals at `rate`
    per second for `duration` seconds; each request 1-500 guides (log-uniform)
    with PAM family and editor drawn as in the batched config, max_mismatches
    uniform in 3..5."""
    from beguidedoff_gb300.types import GuideInput

    rng = np.random.default_rng(seed)
    fams = [p for p, _ in MIXED_FAMILIES]
    probs = np.array([f for _, f in MIXED_FAMILIES])
    t, out = 0.0, []
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t > duration:
            return out
        n = int(np.exp(rng.uniform(0, np.log(500))))
        k = int(rng.integers(3, 6))
        guides = []
        for j in range(n):
            ed = ("ABE", 4, 8, "ABE8e") if rng.random() < 0.5 else ("CBE", 4, 8, "TadCBEd")
            guides.append(GuideInput(f"g{j}", "".join(rng.choice(list("ACGT"), 20)),
                                     fams[int(rng.choice(len(fams), p=probs))], "3prime",
                                     ed[1], ed[2], ed[0], base_editor=ed[3]))
        out.append((t, guides, k))


def _latency_stats(lat, wall, n_guides, comps):
    lat = np.sort(np.asarray(lat))
    return {"requests": int(lat.size), "p50_ms": 1e3 * float(np.percentile(lat, 50)),
            "p99_ms": 1e3 * float(np.percentile(lat, 99)), "mean_ms": 1e3 * float(lat.mean()),
            "max_ms": 1e3 * float(lat.max()), "wall_s": wall,
            "requests_per_s": lat.size / wall, "guides_per_s": n_guides / wall,
            "cmp_per_s": comps / wall}


def _table_rows(t):
    return [dict(r) for r in t.rows()] if hasattr(t, "rows") else t.to_dict("records")


def serve_run(genome, total, local, rate, duration, slots, memory_gb, batch_guides,
              baselines=("same_kernel", "brute_force")):
    """A seeded request trace through the continuous-batching server, then
    through serial per-request search() calls on the same trace: in the
    server's own autotuned forms (same_kernel: the server's finder, one request
    at a time) and, optionally, in the brute-force form (scan mode 0)."""
    from beguidedoff_gb300.finder import beguidedoff
    from beguidedoff_gb300.serving import SearchServer

    trace = serve_trace(rate, duration)
    warm = serve_trace(rate, min(3.0, duration), seed=99)
    n_guides = sum(len(g) for _, g, _ in trace)
    comps = n_guides * 2 * (total - 26)

    def replay_server(srv, items):
        t0 = time.perf_counter()
        done_at = {}
        futs = []
        for i, (t, guides, k) in enumerate(items):
            d = t0 + t - time.perf_counter()
            if d > 0:
                time.sleep(d)
            fut = srv.submit(guides, k)
            fut.add_done_callback(lambda f, i=i: done_at.__setitem__(i, time.perf_counter()))
            futs.append(fut)
        res = [f.result() for f in futs]
        wall = time.perf_counter() - t0
        lat = [done_at[i] - (t0 + items[i][0]) for i in range(len(items))]
        return lat, wall, res

    def replay_serial(fin, items):
        t0 = time.perf_counter()
        lat, res = [], []
        for t, guides, k in items:
            d = t0 + t - time.perf_counter()
            if d > 0:
                time.sleep(d)
            fin.max_mismatches = k
            res.append(fin.search(guides=guides, verbose=False))
            lat.append(time.perf_counter() - (t0 + t))
        return lat, time.perf_counter() - t0, res

    srv = SearchServer(genome_data=genome, device=f"cuda:{local}", n_slots=slots,
                       memory_bytes=memory_gb << 30, max_batch_guides=batch_guides)
    t_tune = time.perf_counter()
    srv.warmup()
    t_tune = time.perf_counter() - t_tune
    replay_server(srv, warm)
    b0 = len(srv.batches)
    x0 = [e.transfer() for e, _ in srv.slots]
    lat_b, wall_b, res_b = replay_server(srv, trace)
    x1 = [e.transfer() for e, _ in srv.slots]
    batches = srv.batches[b0:]
    launches = sum(e.launch_count() for e, _ in srv.slots)
    srv_stats = _latency_stats(lat_b, wall_b, n_guides, comps)
    srv_stats.update({
        "batches": len(batches),
        "requests_per_batch": float(np.mean([b["requests"] for b in batches])),
        "guides_per_batch": float(np.mean([b["guides"] for b in batches])),
        "slots": slots, "memory_gb": memory_gb,
        "max_batch_guides": batch_guides, "tuning_warmup_s": t_tune,
        "batch_seconds": {k: float(np.mean([b.get(k, 0.0) for b in batches]))
                          for k in ("seconds", "plan_s", "scan_s", "epilogue_s", "assemble_s")},
        "autotune": {f"k{k[0]}/size{k[1]}": v.name for k, v in
                     (srv.finder._tuner.cache.items() if srv.finder._tuner else [])}})
    serial = {}
    same = True
    # serial, one request at a time, in the server's own tuned forms
    if "same_kernel" in baselines:
        replay_serial(srv.finder, warm[:4])
        lat_s, wall_s, res_s = replay_serial(srv.finder, trace)
        serial["same_kernel"] = _latency_stats(lat_s, wall_s, n_guides, comps)
        same = same and all(_table_rows(a) == _table_rows(b) for a, b in zip(res_b, res_s))
    srv.close()
    if "brute_force" in baselines:
        base = beguidedoff(None, max_mismatches=4, genome_data=genome, device=f"cuda:{local}",
                           scan_mode=0)
        replay_serial(base, warm[:4])
        lat_s, wall_s, res_s = replay_serial(base, trace)
        base.close()
        serial["brute_force"] = _latency_stats(lat_s, wall_s, n_guides, comps)
        same = same and all(_table_rows(a) == _table_rows(b) for a, b in zip(res_b, res_s))
    h2d = sum(b["h2d"] - a["h2d"] for a, b in zip(x0, x1))
    d2h = sum(b["d2h"] - a["d2h"] for a, b in zip(x0, x1))
    out = {"requests": len(trace), "guides": n_guides, "rate_per_s": rate,
           "duration_s": duration, "serving": srv_stats, "serial": serial,
           "results_identical": same, "gpu_launches": launches,
           "h2d_bytes_per_request": h2d // max(1, len(trace)),
           "d2h_bytes_per_request": d2h // max(1, len(trace))}
    for name, st in serial.items():
        out[f"p50_speedup_vs_serial_{name}"] = st["p50_ms"] / srv_stats["p50_ms"]
        out[f"p99_speedup_vs_serial_{name}"] = st["p99_ms"] / srv_stats["p99_ms"]
    return out


def bench_serve(args, ws, rank, local):
    """Serving loop: the same request trace through the continuous-batching
    server and through serial per-request search() calls (the server's own
    tuned forms, and the brute-force form)."""
    from beguidedoff_gb300 import _native, build

    build.build()
    lens, blocks, _ = make_workload(args.genome_bp, 1)
    total = int(lens.sum())
    genome = _native.synth_genome(7, lens, blocks, thresholds=(76, 128, 180), device=local)
    clocks = ClockSampler(local).start()
    r = serve_run(genome, total, local, args.rate, args.duration, args.slots, args.serve_memory,
                  args.batch_guides)
    clk = clocks.stop()
    st = r["serving"]
    out = {
        "metric": METRIC, "value": st["cmp_per_s"], "unit": UNIT, "n_gpus": ws,
        "steps": r["requests"], "warmup": 0, "ms_per_step": st["mean_ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic",
        "config": {"workload": (f"serving loop: synthetic {total / 1e9:.2f} Gbp resident, Poisson "
                                f"arrivals at {args.rate} req/s for {args.duration} s, 1-500 "
                                f"guides per request (log-uniform), PAM families and editors as "
                                f"the batched config, max_mismatches 3-5; a step = one request"),
                   "genome_bp": total, "requests": r["requests"], "guides": r["guides"],
                   "rate_per_s": args.rate, "duration_s": args.duration,
                   "l2": "inputs larger than L2 (bit planes of both strands ~2.3 GB)"},
        **{k: v for k, v in r.items() if k not in ("requests", "guides")},
        "e2e": {"value": st["cmp_per_s"], "unit": UNIT,
                "h2d_bytes_per_step": r["h2d_bytes_per_request"],
                "d2h_bytes_per_step": r["d2h_bytes_per_request"],
                "note": "the genome stays resident; per request: guides, plan and epilogue "
                        "inputs up, epilogue results down"},
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(out))


def sub_mixed(f, lens, blocks, args, sp, timed, n_guides=1000, max_mm=5, steps=3):
    """The batched mixed-PAM record on the genome already resident: 1,000
    guides (NGG 40% NG 20% NNGRRT 15% NNNRRT 15% NRN 10%; the SaCas9 families
    21 nt), max_mismatches 5; the autotuned batched form (one graph replay)
    against the plain forms of plain_forms(), with key sets compared and the
    keys checked against the oracle on sampled ranges."""
    from types import SimpleNamespace

    from beguidedoff_gb300 import _native

    total = int(np.asarray(lens).sum())
    rng = np.random.default_rng(12)
    guides = ["".join(rng.choice(list("ACGT"), 20)) for _ in range(n_guides)]
    pams = []
    for pam, frac in MIXED_FAMILIES:
        pams += [pam] * int(round(frac * n_guides))
    pams = (pams + ["NGG"] * n_guides)[:n_guides]
    guides = sacas9_extend(guides, pams)
    comps = n_guides * 2 * (total - 26)
    eng, st = f._engine, f._strands
    plan = f._plan(guides, pams)
    try:
        t0 = time.perf_counter()
        mode = f._mode_for(plan, pams, max_mm)
        tune_s = time.perf_counter() - t0
        choice = f.last_choice
        forms = plain_forms(f, plan, pams, SimpleNamespace(max_mm=max_mm), sp, timed, comps,
                            steps)
        if mode in (2, 3):
            g = _native.Graph(eng, plan, st, [0, 3], max_mm, mode)
            step = lambda: g.replay(sp)  # noqa: E731
        else:
            g = None
            step = lambda: eng.launch(plan, st, [0, 3], max_mm, mode, sp)  # noqa: E731
        step()
        eng.complete(plan, st, [0, 3], max_mm, mode, sp)
        _, tot = timed(step, steps)
        n, keys = eng.collect(sp)
        if g is not None:
            g.close()
        batched_ms = tot / steps
        for form in forms.values():
            k = form.pop("_k", None)
            form["keys_equal"] = bool(k is not None and keys is not None and
                                      np.array_equal(k, keys))
        out = {"workload": (f"batched mixed-PAM scan on the resident {total / 1e9:.2f} Gbp "
                            f"genome: {n_guides} guides (NGG 40% NG 20% NNGRRT 15% NNNRRT 15% "
                            f"NRN 10%, SaCas9 guides 21 nt), max_mismatches {max_mm}, both strands"),
               "guides": n_guides, "max_mismatches": max_mm,
               "batched": {"form": choice.name if choice else str(mode), "graph": g is not None,
                           "ms_per_step": batched_ms, "value": comps / (batched_ms / 1e3),
                           "hits_per_step": n},
               "autotune_s": tune_s, "autotune": choice.as_dict() if choice else None,
               "plain_forms": forms, **speedups(forms, batched_ms)}
        if not args.no_cpu and keys is not None:
            out["parity"] = range_parity(
                [(f._strand_arrays[0], f._n_mask_fwd, 0), (f._strand_arrays[1], f._n_mask_rc, 3)],
                total, guides, pams, max_mm, keys, sampled_ranges(lens, blocks, 4, 1_000_000))
        return out
    finally:
        plan.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="auto", choices=["auto", "0", "1", "2", "3"],
                    help="scan form: auto = the project autotuner's choice")
    ap.add_argument("--chunk-sites", type=int, default=0, help="modes 2/3 tile length (0 = default)")
    ap.add_argument("--group-guides", type=int, default=0, help="mode 3 guides per group")
    ap.add_argument("--ctas-per-sm", type=int, default=0)
    ap.add_argument("--min-blocks", type=int, default=0,
                    help="mode 2: 3 or 4 CTAs of 256 threads per SM; 1 = one of 768, "
                         "2 = one of 512")
    ap.add_argument("--tolerance", type=int, default=0, help="mode 2: key-region tolerance 0/1")
    ap.add_argument("--split-families", type=int, default=0, help="mode 2: one launch per family")
    ap.add_argument("--inline-entries", type=int, default=0, help="mode 2: 1 or 2 inline guides")
    ap.add_argument("--range-walk", type=int, default=0, help="mode 2: per-lane walk of buckets")
    ap.add_argument("--prefilter", type=int, default=0,
                    help="mode 2: the prefiltered form (tolerance 1; chunk sites 2048|4096)")
    ap.add_argument("--genome-bp", type=int, default=3_100_000_000)
    ap.add_argument("--guides", type=int, default=100)
    ap.add_argument("--max-mm", type=int, default=4)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-subrecords", action="store_true",
                    help="plain config: skip the mixed-PAM 1,000-guide and serving records")
    ap.add_argument("--families", default="", help="mixed/dense: keep only these PAM families "
                                                   "(comma list), e.g. NRN")
    ap.add_argument("--rate", type=float, default=20.0, help="serve: requests per second")
    ap.add_argument("--duration", type=float, default=15.0, help="serve: trace seconds")
    ap.add_argument("--slots", type=int, default=2, help="serve: concurrent batches")
    ap.add_argument("--serve-memory", type=int, default=16, help="serve: output-buffer GB")
    ap.add_argument("--batch-guides", type=int, default=2048, help="serve: guides per batch")
    ap.add_argument("--config", default="plain", choices=["plain", "mixed", "dense", "serve"],
                    help="plain: 100 NGG guides, <=4 mm; mixed: 400 mixed-PAM guides, <=5 mm; "
                         "dense: repeat-family genome, 1000 mixed guides, <=6 mm")
    args = ap.parse_args()
    args.mode_requested = args.mode
    if args.mode != "auto":
        args.mode = int(args.mode)
    if args.warmup < 3:
        args.warmup = 3
    if args.config in ("mixed", "dense"):
        if "--guides" not in sys.argv:
            args.guides = 400 if args.config == "mixed" else 1000
        if "--max-mm" not in sys.argv:
            args.max_mm = 5 if args.config == "mixed" else 6
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        bench_reference(args, ws, rank)
    elif args.config == "serve":
        bench_serve(args, ws, rank, local)
    else:
        bench_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
