"""ORACLE: CPU restatement of the reference's extensive search (test infrastructure).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline /
reference arm may import this module, and only as the checker or the timed CPU
baseline.  The product (``beguidedoff_gb300``) never imports it.

Contents
--------
* ``scan_strand``: ctypes front end of ``scan_oracle.c``, the C restatement of
  ``search_chunk_kernel`` (beguidedoff/cuda_search.py:163-314).
* ``search_genome_seam``: the reference's kernel driver contract
  (beguidedoff/cuda_search.py:384-488): per guide the first
  ``results_per_guide`` hits, an overflow flag and the exact count.
* ``bruteforce_strand``: an independent NumPy formulation of the same scan
  (per-base arrays and sliding windows instead of packed words), for small
  genomes; it cross-checks ``scan_oracle.c``.
* ``prepare_n_masks``: beguidedoff/finder.py:310-345.
* ``oracle_search``: the finder's host logic in plain Python loops
  (beguidedoff/finder.py:119-249, :361-472, :474-566, :568-679), returning the
  output table as a list of row dicts with the reference's columns.

Parity pin: tests/test_oracle_golden.py checks ``scan_strand`` and
``oracle_search`` against the outputs recorded from the reference itself
(tests/golden/*.npz, made by tests/golden/make_golden.py).
"""
import ctypes
import logging
import os
import subprocess
from collections import defaultdict

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD_DIR = os.path.join(HERE, "_build")
_LIB_PATH = os.path.join(_BUILD_DIR, "liboracle.so")
_SRC = os.path.join(HERE, "scan_oracle.c")
_LIB = None

MAX_PAM_LEN = 6
BIT_TO_NUC = "ACGT"
IUPAC_MASK = {"A": 1, "C": 2, "G": 4, "T": 8, "R": 5, "Y": 10, "M": 3, "K": 12, "S": 6,
              "W": 9, "H": 11, "B": 14, "V": 7, "D": 13, "N": 15}
_EDIT_TARGET = {"CBE": "C", "ABE": "A", "CGE": "C"}


# ----------------------------------------------------------------------------
# C oracle
# ----------------------------------------------------------------------------
def build(force=False):
    """Compile scan_oracle.c into oracle/_build/liboracle.so (gcc, OpenMP)."""
    os.makedirs(_BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(_SRC)):
        return _LIB_PATH
    cmd = ["gcc", "-O2", "-fopenmp", "-shared", "-fPIC", "-std=c11", _SRC, "-o", _LIB_PATH]
    subprocess.run(cmd, check=True)
    return _LIB_PATH


def _lib():
    global _LIB
    if _LIB is None:
        build()
        lib = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        i32 = ctypes.c_int32
        lib.oracle_scan_strand.argtypes = [P, i64, i64, P, i64, P, P, P, P, i32, i32, i32,
                                           i64, i64, ctypes.c_int, P,
                                           ctypes.POINTER(ctypes.c_void_p),
                                           ctypes.POINTER(i64)]
        lib.oracle_scan_strand.restype = ctypes.c_int
        lib.oracle_free.argtypes = [P]
        lib.oracle_max_threads.restype = ctypes.c_int
        _LIB = lib
    return _LIB


def max_threads():
    return int(_lib().oracle_max_threads())


def _ptr(a):
    return a.ctypes.data if a is not None and a.size else None


def scan_strand(packed, total_bp, n_mask_le, guides, pam_masks, pam_lens, pam_3prime,
                max_mismatches, n_encoded, pos_begin=0, pos_end=None, n_threads=0):
    """Scan one strand array; returns (counts int64[n], keys uint64[h]).

    Keys are ``guide << 40 | pos << 5 | mm`` sorted ascending.  ``n_mask_le``
    is the padded little-bit-order mask or None (no N gating).
    """
    packed = np.ascontiguousarray(packed, dtype=np.uint32)
    guides = np.ascontiguousarray(guides, dtype=np.uint64)
    n = int(guides.size)
    pm = np.zeros((n, MAX_PAM_LEN), dtype=np.uint8)
    if n:
        src = np.asarray(pam_masks, dtype=np.uint8).reshape(n, -1)
        pm[:, :min(src.shape[1], MAX_PAM_LEN)] = src[:, :MAX_PAM_LEN]
    pl = np.ascontiguousarray(pam_lens, dtype=np.uint8)
    p3 = np.ascontiguousarray(pam_3prime, dtype=np.uint8)
    nm = None if n_mask_le is None else np.ascontiguousarray(n_mask_le, dtype=np.uint8)
    counts = np.zeros(max(n, 1), dtype=np.int64)
    kp = ctypes.c_void_p()
    nk = ctypes.c_int64()
    end = int(total_bp) if pos_end is None else int(pos_end)
    rc = _lib().oracle_scan_strand(
        _ptr(packed), packed.size, int(total_bp), _ptr(nm), 0 if nm is None else nm.size,
        _ptr(guides), _ptr(pm), _ptr(pl), _ptr(p3), n, int(max_mismatches), int(n_encoded),
        int(pos_begin), end, int(n_threads), counts.ctypes.data, ctypes.byref(kp),
        ctypes.byref(nk))
    if rc != 0:
        raise MemoryError("oracle scan failed")
    keys = np.empty(nk.value, dtype=np.uint64)
    if nk.value:
        ctypes.memmove(keys.ctypes.data, kp.value, nk.value * 8)
    if kp.value:
        _lib().oracle_free(kp)
    return counts[:n], keys


def split_keys(keys):
    keys = np.asarray(keys, dtype=np.uint64)
    return ((keys >> np.uint64(40)).astype(np.int64),
            ((keys >> np.uint64(5)) & np.uint64((1 << 35) - 1)).astype(np.int64),
            (keys & np.uint64(31)).astype(np.int64))


def search_genome_seam(packed, total_bp, guides, pam_masks, pam_lens, pam_3prime,
                       max_mismatches, results_per_guide, n_mask_le, n_encoded):
    """The reference driver contract (cuda_search.py:384-488) on the C oracle.

    Returns (results {g: [(pos, mm), ...]}, overflow {g: bool}, counts {g: int});
    each list holds the first ``results_per_guide`` hits in genome order.
    """
    counts, keys = scan_strand(packed, total_bp, n_mask_le, guides, pam_masks, pam_lens,
                               pam_3prime, max_mismatches, n_encoded)
    g, pos, mm = split_keys(keys)
    res = {i: [] for i in range(len(counts))}
    for gi, p, m in zip(g.tolist(), pos.tolist(), mm.tolist()):
        if len(res[gi]) < results_per_guide:
            res[gi].append((p, m))
    ovf = {i: int(c) > results_per_guide for i, c in enumerate(counts)}
    cnt = {i: int(c) for i, c in enumerate(counts)}
    return res, ovf, cnt


# ----------------------------------------------------------------------------
# NumPy brute force (independent formulation, small genomes)
# ----------------------------------------------------------------------------
def unpack_bases(packed, total_bp):
    packed = np.asarray(packed, dtype=np.uint32)
    shifts = (np.arange(16, dtype=np.uint32) * 2)[None, :]
    return ((packed[:, None] >> shifts) & 3).astype(np.uint8).reshape(-1)[:total_bp]


def bruteforce_strand(packed, total_bp, n_mask_le, guide_seqs_2bit, pam_masks, max_mismatches,
                      n_encoded):
    """3' PAM scan of one strand from per-base arrays; returns a set of
    (guide, pos, mm).  ``guide_seqs_2bit`` is uint8[n, 20]."""
    bases = unpack_bases(packed, total_bp)
    nbits = np.zeros(total_bp, dtype=bool)
    if n_mask_le is not None:
        nb = np.unpackbits(np.asarray(n_mask_le, dtype=np.uint8), bitorder="little")
        k = min(nb.size, total_bp)
        nbits[:k] = nb[:k].astype(bool)
    n_sites = total_bp - 26
    out = set()
    if n_sites <= 0:
        return out
    idx = np.arange(n_sites)[:, None] + np.arange(26)[None, :]
    win = bases[idx]                     # [sites, 26]
    nwin = nbits[idx[:, :20]]
    for g in range(len(guide_seqs_2bit)):
        masks = np.asarray(pam_masks[g], dtype=np.uint8)
        plen = int(np.count_nonzero(masks))
        ok = np.ones(n_sites, dtype=bool)
        for i in range(plen):
            ok &= ((np.uint8(1) << win[:, 20 + i]) & masks[i]) != 0
        gs = np.asarray(guide_seqs_2bit[g], dtype=np.uint8)
        raw = (win[:, :20] != gs[None, :]).sum(axis=1)
        extra = (nwin & (gs[None, :] == n_encoded)).sum(axis=1)
        mm = raw + extra
        hit = ok & (raw <= max_mismatches) & (mm <= max_mismatches)
        for p in np.nonzero(hit)[0].tolist():
            out.add((g, p, int(mm[p])))
    return out


# ----------------------------------------------------------------------------
# Host logic of the finder (plain Python)
# ----------------------------------------------------------------------------
def prepare_n_masks(genome):
    """beguidedoff/finder.py:310-345: (fwd, rc) little-bit-order masks, padded
    by 16 bytes, or (None, None) when the genome has no N."""
    packed_big = genome.get("n_mask")
    total_bp = int(genome["total_bp"])
    if packed_big is None or np.asarray(packed_big).size == 0:
        return None, None
    bits = np.unpackbits(np.asarray(packed_big, dtype=np.uint8), bitorder="big", count=total_bp)
    if not bits.any():
        return None, None
    fwd = np.pad(np.packbits(bits, bitorder="little"), (0, 16))
    rc_bits = np.empty(total_bp, dtype=np.uint8)
    for off, ln in zip(genome["chrom_offsets"], genome["chrom_lengths"]):
        off, ln = int(off), int(ln)
        rc_bits[off:off + ln] = bits[off:off + ln][::-1]
    rc = np.pad(np.packbits(rc_bits, bitorder="little"), (0, 16))
    return fwd, rc


def encode_guide(seq):
    v = 0
    for i, c in enumerate(seq.upper()):
        v |= {"A": 0, "C": 1, "G": 2, "T": 3}.get(c, 0) << (2 * i)
    return v


def _chrom_index(pos, offsets):
    """np.searchsorted(offsets, pos, 'right') - 1, including the reference's
    wrap to the last chromosome for a negative position (Python indexing)."""
    idx = int(np.searchsorted(offsets, pos, side="right") - 1)
    return idx, int(pos - offsets[idx])


def _decode(packed, start, n):
    out = []
    for i in range(n):
        p = start + i
        out.append(BIT_TO_NUC[(int(packed[p // 16]) >> ((p % 16) * 2)) & 3])
    return "".join(out)


def _mismatch_positions(gval, wval):
    x = gval ^ wval
    m = (x | (x >> 1)) & 0x5555555555
    return [i + 1 for i in range(20) if (m >> (2 * i)) & 1]


def _cctop(positions):
    if not positions:
        return 0.0
    return sum(1.2 ** p for p in positions)


def _editable(seq, editor_type, ws, we):
    tb = _EDIT_TARGET.get(editor_type)
    if tb is None:
        raise ValueError(f"Unknown editor_type: {editor_type}")
    return [i + 1 for i in range(ws - 1, we) if i < len(seq) and seq[i] == tb]


def oracle_search(genome, guides, max_mismatches=4, n_top_offtargets=3,
                  results_per_guide=10240, max_results_per_guide=2_621_440,
                  return_all=False, count_score_threshold=None, log=None):
    """Extensive search on the C oracle with the reference's host semantics.

    ``genome``: dict with the .npz keys; ``guides``: sequence of objects with
    the ``GuideInput`` attributes.  Returns the output rows (list of dicts).
    """
    log = log or logging.getLogger("oracle")
    names = [str(c) for c in genome["chrom_names"]]
    offsets = np.asarray(genome["chrom_offsets"], dtype=np.int64)
    lengths = np.asarray(genome["chrom_lengths"], dtype=np.int64)
    total_bp = int(genome["total_bp"])
    nm_fwd, nm_rc = prepare_n_masks(genome)
    for g in guides:
        if g.pam_position.lower() != "3prime":
            raise ValueError("Only 3prime PAM is supported.")
    # dedup (finder.py:361-403)
    mapping = defaultdict(list)
    for g in guides:
        ot = (None, None, None)
        if g.on_target_chrom and g.on_target_pos is not None:
            ci = names.index(g.on_target_chrom) if g.on_target_chrom in names else None
            if ci is not None:
                if g.on_target_strand is None:
                    raise ValueError("on-target chromosome and position but no strand")
                w = 20 + len(g.pam)
                lp = g.on_target_pos - 1 if g.on_target_strand == "+" else g.on_target_pos - w
                ot = (ci, lp, g.on_target_strand)
        mapping[(g.guide_seq, g.pam) + ot].append(g)
    keys = list(mapping)
    n = len(keys)
    gv = np.array([encode_guide(k[0]) for k in keys], dtype=np.uint64)
    pm = np.zeros((n, MAX_PAM_LEN), dtype=np.uint8)
    for i, k in enumerate(keys):
        for j, c in enumerate(k[1].upper()):
            pm[i, j] = IUPAC_MASK[c]
    pl = np.array([len(k[1]) for k in keys], dtype=np.uint8)
    p3 = np.ones(n, dtype=np.uint8)
    strands = [("+", genome["genome_forward"], nm_fwd, 0)]
    if "genome_rc" in genome:
        strands.append(("-", genome["genome_rc"], nm_rc, 3))
    # exact per-strand hits, then the re-scan escalation of finder.py:568-638
    per_strand = []
    for label, arr, nm, ne in strands:
        counts, hk = scan_strand(arr, total_bp, nm, gv, pm, pl, p3, max_mismatches, ne)
        per_strand.append((label, arr, counts, split_keys(hk)))
    cap = max_results_per_guide
    limit = {}
    truncated = []
    for i in range(n):
        rpg = results_per_guide
        while True:
            over = any(int(c[i]) > rpg for _l, _a, c, _h in per_strand)
            if not over:
                break
            if rpg >= cap:
                truncated.append(i)
                break
            rpg = min(rpg * 16, cap)
        limit[i] = rpg
    for i in sorted(truncated, key=lambda j: keys[j][0]):
        tot = sum(int(c[i]) for _l, _a, c, _h in per_strand)
        log.warning("Truncated off-target enumeration for guide %s (PAM=%s): %d raw "
                    "genome-wide hits exceed the per-strand buffer of %d", keys[i][0],
                    keys[i][1], tot, limit[i])
    # raw hit decode (finder.py:193-244)
    raw = {i: [] for i in range(n)}
    for label, arr, counts, (hg, hp, hm) in per_strand:
        taken = defaultdict(int)
        for gi, pos, mm in zip(hg.tolist(), hp.tolist(), hm.tolist()):
            if taken[gi] >= limit[gi]:
                continue
            taken[gi] += 1
            plen = len(keys[gi][1])
            win = 20 + plen
            if label == "+":
                leftmost = pos
                report = pos
            else:
                ci, local_rc = _chrom_index(pos, offsets)
                leftmost = int(offsets[ci] + (lengths[ci] - local_rc - win))
                report = leftmost + win - 1
            ot_ci, ot_lp, ot_st = keys[gi][2:]
            if ot_ci is not None:
                ci, local = _chrom_index(leftmost, offsets)
                if ci == ot_ci and local == ot_lp and label == ot_st:
                    continue
            raw[gi].append((report, mm, _decode(arr, pos, 20), _decode(arr, pos + 20, plen),
                            label))
    # scoring, editable filter, thresholds (finder.py:405-472)
    include_non_editable = return_all
    groups = defaultdict(list)
    below = defaultdict(int)
    for gi, hits in raw.items():
        gval = int(gv[gi])
        for report, mm, seq, pam, label in hits:
            ci, local = _chrom_index(report, offsets)
            mpos = _mismatch_positions(gval, encode_guide(seq))
            score = _cctop(mpos)
            for g in mapping[keys[gi]]:
                ed = _editable(seq, g.editor_type, g.edit_window_start, g.edit_window_end)
                if not include_non_editable and not ed:
                    continue
                groups[g.guide_id].append(dict(
                    chromosome=names[ci], position=local + 1, strand=label, seq=seq, pam=pam,
                    guide_seq=keys[gi][0], base_editor=g.base_editor or "", n_mm=mm,
                    mpos=mpos, score=score))
                if count_score_threshold is not None and ed and score <= count_score_threshold:
                    below[g.guide_id] += 1
    # sort, top-N, table (finder.py:545-566, io.py:155-180)
    rows = []
    for g in guides:
        hits = groups.get(g.guide_id, [])
        hits.sort(key=lambda h: (h["score"], h["chromosome"], h["position"], h["strand"]))
        if not return_all:
            hits = hits[:n_top_offtargets]
        for rank, h in enumerate(hits, start=1):
            rows.append({
                "guide_rna_sequence": h["guide_seq"], "base_editor": h["base_editor"],
                "ot_rank": rank, "ot_chromosome": h["chromosome"], "ot_position": h["position"],
                "ot_strand": h["strand"], "ot_sequence": h["seq"], "ot_pam": h["pam"],
                "n_mismatches": h["n_mm"],
                "mismatch_positions": ",".join(map(str, h["mpos"])),
                "score": round(h["score"], 6),
                "n_offtargets_below_threshold": below.get(g.guide_id, 0),
            })
    return rows
