"""The kernel-driver seam: ``search_genome_cuda`` with the reference's signature
and return values (beguidedoff/cuda_search.py:384-488), running the sm_103a scan
through the C ABI (``bgo_search_genome``).

Differences from the reference, by design:
  * there is no chunk loop (``chunk_size`` is accepted and ignored): one launch
    per PAM family covers the strand;
  * each guide's recorded hits are its first ``results_per_guide`` hits in
    genome order (the reference keeps them in atomic-append order);
  * ``MAX_GUIDES`` is kept for callers that batch by it, with the reference's
    error above it, although the device plan has no shared-memory limit.
"""
import numpy as np

from . import _native

MAX_GUIDES = 2048
MAX_PAM_LEN = 6
_DEFAULT_RESULTS_PER_GUIDE = 10240

_ENGINES = {}
_STRANDS = {}
_CACHE_LIMIT = 4


def _pam_nibble_fields(nib):
    """Packed (pattern, compare) bits of one IUPAC nibble, or None when the
    allowed set is not a fixed-bit pattern (beguidedoff/cuda_search.py:101-121)."""
    bases = [b for b in range(4) if nib & (1 << b)]
    if len(bases) == 1:
        return bases[0], 0b11
    if len(bases) == 4:
        return 0, 0b00
    if len(bases) == 2:
        lo, hi = bases
        if (lo & 1) == (hi & 1) and (lo >> 1) != (hi >> 1):
            return lo & 1, 0b01
        if (lo >> 1) == (hi >> 1) and (lo & 1) != (hi & 1):
            return lo & 2, 0b10
    return None


def encode_pam_packed(pam_masks, pam_lens, pam_3prime):
    """The reference's packed PAM fields (beguidedoff/cuda_search.py:124-160),
    kept for API compatibility; the device plan uses the allowed-set nibbles."""
    n = int(np.asarray(pam_masks).shape[0])
    pats = np.zeros(n, dtype=np.uint32)
    cmps = np.zeros(n, dtype=np.uint32)
    for g in range(n):
        plen = int(pam_lens[g])
        if plen == 0 or plen > MAX_PAM_LEN:
            continue
        pat = cmp_mask = 0
        exotic = False
        for i in range(plen):
            res = _pam_nibble_fields(int(pam_masks[g][i]) & 0xF)
            if res is None:
                exotic = True
                break
            pat |= res[0] << (2 * i)
            cmp_mask |= res[1] << (2 * i)
        info = (pat & 0xFFF) | (plen << 12)
        if exotic:
            info |= 1 << 15
            cmp_mask = 0
        if pam_3prime[g]:
            info |= 1 << 16
        pats[g] = info
        cmps[g] = cmp_mask
    return pats, cmps


def _engine(device):
    e = _ENGINES.get(device)
    if e is None:
        e = _ENGINES[device] = _native.Engine(device)
    return e


def _strand(genome_packed, total_bp, n_mask_packed, device):
    """Device copy of a strand, cached by the identity of the host arrays."""
    key = (id(genome_packed), id(n_mask_packed), int(total_bp), device)
    hit = _STRANDS.get(key)
    if hit is not None and hit[0] is genome_packed and hit[1] is n_mask_packed:
        return hit[2]
    if len(_STRANDS) >= _CACHE_LIMIT:
        _STRANDS.clear()
    nm = None
    if n_mask_packed is not None and np.asarray(n_mask_packed).size:
        nm = np.asarray(n_mask_packed, dtype=np.uint8)
    s = _native.Strand(genome_packed, total_bp, nm, device)
    _STRANDS[key] = (genome_packed, n_mask_packed, s)
    return s


def search_genome_cuda(genome_packed, total_bp, guide_encoded, pam_masks, pam_lens, pam_3prime,
                       max_mismatches, chunk_size=200_000_000, return_overflow=False,
                       results_per_guide=_DEFAULT_RESULTS_PER_GUIDE, n_mask_packed=None,
                       n_encoded=0, device=0):
    """Scan one strand array.  Returns {guide: [(position, mismatches), ...]},
    and with return_overflow also {guide: bool} and {guide: exact count}."""
    ng = len(guide_encoded)
    if ng > MAX_GUIDES:
        raise RuntimeError(
            f"Too many guides ({ng}) for GPU search. Maximum supported is {MAX_GUIDES}. "
            f"Consider splitting the input into smaller batches, "
            f"or increase MAX_GUIDES in cuda_search.py.")
    engine = _engine(device)
    strand = _strand(genome_packed, total_bp, n_mask_packed, device)
    gv = np.ascontiguousarray(guide_encoded, dtype=np.uint64)
    pm = np.zeros((ng, 6), dtype=np.uint8)
    if ng:
        src = np.asarray(pam_masks, dtype=np.uint8).reshape(ng, -1)
        pm[:, :min(6, src.shape[1])] = src[:, :6]
    pl = np.ascontiguousarray(pam_lens, dtype=np.uint8)
    p3 = np.ascontiguousarray(pam_3prime, dtype=np.uint8)
    rpg = int(results_per_guide)
    counts = np.zeros(max(ng, 1), dtype=np.int64)
    hp = np.zeros(max(ng * rpg, 1), dtype=np.int64)
    hm = np.zeros(max(ng * rpg, 1), dtype=np.int8)
    _native.check(_native.lib().bgo_search_genome(
        engine.handle, strand.handle, _native.ptr(gv), _native.ptr(pm), _native.ptr(pl),
        _native.ptr(p3), ng, int(max_mismatches), int(n_encoded), rpg, counts.ctypes.data,
        hp.ctypes.data, hm.ctypes.data, None), "bgo_search_genome")
    results, overflow, hit_counts = {}, {}, {}
    for g in range(ng):
        c = int(counts[g])
        k = min(c, rpg)
        results[g] = list(zip(hp[g * rpg:g * rpg + k].tolist(), hm[g * rpg:g * rpg + k].tolist()))
        overflow[g] = c > rpg
        hit_counts[g] = c
    if return_overflow:
        return results, overflow, hit_counts
    return results
