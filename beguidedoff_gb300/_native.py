"""ctypes bindings of the native library (include/bgo.h).

The library is built in-tree (``beguidedoff_gb300/_build/libbgo.so``) by
``beguidedoff_gb300.build.build()``.  There is no CPU fallback: if the
library is missing, every GPU entry point raises ``NativeLibraryMissing``.
"""
import ctypes
import os

import numpy as np

from . import build as _build

BGO_OK = 0
BGO_ERR_ARG = -1
BGO_ERR_CUDA = -2
BGO_ERR_OOM = -3
BGO_ERR_TIMEOUT = -4
BGO_ERR_STATE = -5

# Names of every function declared in include/bgo.h.
EXPORTED = [
    "bgo_version", "bgo_last_error", "bgo_device_count", "bgo_host_alloc", "bgo_host_free",
    "bgo_genome_create", "bgo_genome_destroy", "bgo_genome_info", "bgo_engine_create",
    "bgo_engine_destroy", "bgo_plan_create", "bgo_plan_destroy", "bgo_plan_info",
    "bgo_scan_launch", "bgo_scan_collect", "bgo_engine_reserve", "bgo_search_genome",
    "bgo_engine_info", "bgo_scan_stats",
    "bgo_scan_noalloc", "bgo_graph_create", "bgo_graph_launch", "bgo_graph_destroy",
    "bgo_epilogue_run", "bgo_engine_transfer",
    "bgo_plan_set_tuning", "bgo_epilogue_fetch", "bgo_scan_time", "bgo_stream_create",
    "bgo_stream_destroy", "bgo_plan_families", "bgo_plan_set_family_tuning",
    "bgo_genome_upload", "bgo_encode_genome", "bgo_scan_complete",
]

# Names of every function declared in include/bgo_tools.h (libbgo_tools.so).
TOOLS_EXPORTED = ["bgo_synth_genome", "bgo_synth_genome_repeats", "bgo_probe_int_throughput"]

INPUT_ROW_DTYPE = np.dtype([("plan_row", "<i4"), ("window_mask", "<u4"), ("target_base", "<i4"),
                            ("ot_chrom", "<i4"), ("ot_local", "<i8"), ("ot_strand", "<i4"),
                            ("threshold_rank", "<i4"), ("flags", "<i4"), ("pad", "<i4")])
ROW_RETURN_ALL = 1
RECORD_DTYPE = np.dtype([("key", "<u8"), ("order", "<u8"), ("input_row", "<i4"),
                         ("rank", "<u4")])
assert INPUT_ROW_DTYPE.itemsize == 40 and RECORD_DTYPE.itemsize == 24

NOALLOC_MAX_GUIDES = 2048
NOALLOC_MAX_HITS = 1 << 20


class NativeLibraryMissing(RuntimeError):
    pass


class BgoError(RuntimeError):
    def __init__(self, code, where, message):
        super().__init__(f"{where} failed ({code}): {message}")
        self.code = code


_LIB = None

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_PP = ctypes.POINTER(ctypes.c_void_p)

_SIGS = {
    "bgo_version": ([], ctypes.c_int),
    "bgo_last_error": ([ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
    "bgo_device_count": ([ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "bgo_host_alloc": ([_PP, ctypes.c_size_t], ctypes.c_int),
    "bgo_host_free": ([_P], ctypes.c_int),
    "bgo_genome_create": ([_P, _I64, _I64, _P, _I64, ctypes.c_int, _P, _PP], ctypes.c_int),
    "bgo_genome_destroy": ([_P], ctypes.c_int),
    "bgo_genome_info": ([_P, ctypes.POINTER(_I64), ctypes.POINTER(ctypes.c_int),
                         ctypes.POINTER(_I64)], ctypes.c_int),
    "bgo_engine_create": ([ctypes.c_int, _PP], ctypes.c_int),
    "bgo_engine_destroy": ([_P], ctypes.c_int),
    "bgo_plan_create": ([_P, _P, _P, _P, _P, _I32, _P, _PP], ctypes.c_int),
    "bgo_plan_destroy": ([_P], ctypes.c_int),
    "bgo_plan_info": ([_P, ctypes.POINTER(_I32), ctypes.POINTER(_I32)], ctypes.c_int),
    "bgo_scan_launch": ([_P, _P, _P, _P, _I32, _I32, _I32, _P], ctypes.c_int),
    "bgo_scan_collect": ([_P, _P, _I64, ctypes.POINTER(_I64), _P], ctypes.c_int),
    "bgo_scan_stats": ([_P, ctypes.POINTER(_I64), _P], ctypes.c_int),
    "bgo_graph_create": ([_P, _P, _P, _P, _I32, _I32, _I32, _PP], ctypes.c_int),
    "bgo_graph_launch": ([_P, _P], ctypes.c_int),
    "bgo_graph_destroy": ([_P], ctypes.c_int),
    "bgo_epilogue_run": ([_P, _P, _P, _I32, _P, _I32, _P, _P, _P, _I32, _P, _I32, _P, _P, _P,
                          ctypes.POINTER(_I64), _P], ctypes.c_int),
    "bgo_epilogue_fetch": ([_P, _P, _I64, _P], ctypes.c_int),
    "bgo_stream_create": ([ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "bgo_stream_destroy": ([_P], ctypes.c_int),
    "bgo_plan_families": ([_P, _P], ctypes.c_int),
    "bgo_genome_upload": ([_P, _P, _I64, _P, _I64, _P], ctypes.c_int),
    "bgo_encode_genome": ([_P, _P, _I32, ctypes.c_int, _P, _P, _P], ctypes.c_int),
    "bgo_plan_set_family_tuning": ([_P, _I32, _P], ctypes.c_int),
    "bgo_scan_time": ([_P, _P, _P, _P, _I32, _I32, _I32, _I32, _P,
                       ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    "bgo_scan_noalloc": ([_P, _P, _I32, _P, _P, _P, _P, _I32, _I32, _P, _I64,
                          ctypes.POINTER(_I64), _P], ctypes.c_int),
    "bgo_engine_reserve": ([_P, _I64], ctypes.c_int),
    "bgo_search_genome": ([_P, _P, _P, _P, _P, _P, _I32, _I32, _I32, _I64, _P, _P, _P, _P],
                          ctypes.c_int),
    "bgo_engine_info": ([_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)], ctypes.c_int),
    "bgo_engine_transfer": ([_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)], ctypes.c_int),
    "bgo_plan_set_tuning": ([_P, _P], ctypes.c_int),
    "bgo_scan_complete": ([_P, _P, _P, _P, _I32, _I32, _I32, _P, _P], ctypes.c_int),
    "bgo_synth_genome": ([ctypes.c_uint64, _P, _I32, _P, _P, _I64, _P, ctypes.c_int, _P, _P, _P],
                         ctypes.c_int),
    "bgo_probe_int_throughput": ([ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)],
                                 ctypes.c_int),
    "bgo_synth_genome_repeats": ([ctypes.c_uint64, _P, _I32, _P, _P, _I64, _P, _P, _P,
                                  ctypes.c_int, _P, _P, _P], ctypes.c_int),
}


class RepeatSpec(ctypes.Structure):
    """bgo_repeat_spec."""
    _fields_ = [("n_families", ctypes.c_int32), ("family_len", ctypes.c_int32),
                ("n_copies", ctypes.c_int64), ("divergence_65536", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("seed", ctypes.c_uint64)]


def synth_genome(seed, chrom_lengths, n_blocks=(), thresholds=(64, 128, 192), device=0,
                 out=None, repeats=None):
    """Seeded synthetic genome dict in the reference .npz layout (device
    generator).  ``n_blocks`` = sorted disjoint (start, end) pairs; ``out`` may
    supply preallocated (fwd, rc, n_mask) host arrays, e.g. pinned buffers.
    ``repeats`` = dict(n_families, family_len, n_copies, divergence, seed)
    inserts repeat-family copies; the dict gains ``repeat_families`` (the
    consensus sequences as strings)."""
    lens = np.ascontiguousarray(chrom_lengths, dtype=np.int64)
    total = int(lens.sum())
    nb = np.asarray(list(n_blocks), dtype=np.int64).reshape(-1, 2)
    starts = np.ascontiguousarray(nb[:, 0])
    ends = np.ascontiguousarray(nb[:, 1])
    th = np.ascontiguousarray(thresholds, dtype=np.uint8)
    n_words = (total + 15) // 16
    n_bytes = (total + 7) // 8
    if out is None:
        fwd = np.empty(n_words, dtype=np.uint32)
        rc = np.empty(n_words, dtype=np.uint32)
        nm = np.empty(n_bytes, dtype=np.uint8)
    else:
        fwd, rc, nm = out
        assert fwd.size >= n_words and rc.size >= n_words and nm.size >= n_bytes
    fams = None
    if repeats is None:
        check(tools_lib().bgo_synth_genome(int(seed), ptr(lens), lens.size, ptr(starts), ptr(ends),
                                     starts.size, ptr(th), int(device), fwd.ctypes.data,
                                     rc.ctypes.data, nm.ctypes.data), "bgo_synth_genome")
    else:
        spec = RepeatSpec(int(repeats["n_families"]), int(repeats["family_len"]),
                          int(repeats["n_copies"]),
                          int(round(float(repeats["divergence"]) * 65536)), 0,
                          int(repeats.get("seed", seed)))
        fams = np.zeros(spec.n_families * spec.family_len, dtype=np.uint8)
        check(tools_lib().bgo_synth_genome_repeats(
            int(seed), ptr(lens), lens.size, ptr(starts), ptr(ends), starts.size, ptr(th),
            ctypes.byref(spec), fams.ctypes.data, int(device), fwd.ctypes.data, rc.ctypes.data,
            nm.ctypes.data), "bgo_synth_genome_repeats")
    offsets = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64)
    out = {
        "genome_forward": fwd[:n_words], "genome_rc": rc[:n_words],
        "chrom_names": np.array([f"chr{i + 1}" for i in range(lens.size)]),
        "chrom_offsets": offsets, "chrom_lengths": lens, "total_bp": total,
        "n_mask": nm[:n_bytes],
    }
    if fams is not None:
        out["repeat_families"] = ["".join("ACGT"[b] for b in r)
                                  for r in fams.reshape(spec.n_families, spec.family_len)]
    return out


def encode_genome(seq: bytes, chrom_lengths, include_rc=True, include_n_mask=True, device=0):
    """(forward words, reverse-complement words or None, big-endian N mask or
    None) of concatenated sequence bytes, encoded on the device
    (bgo_encode_genome)."""
    lens = np.ascontiguousarray(chrom_lengths, dtype=np.int64)
    total = int(lens.sum())
    raw = np.frombuffer(seq, dtype=np.uint8) if total else np.zeros(1, dtype=np.uint8)
    if raw.size < total:
        raise ValueError("sequence shorter than the chromosome lengths")
    n_words, n_bytes = (total + 15) // 16, (total + 7) // 8
    fwd = np.zeros(n_words, dtype=np.uint32)
    rc = np.zeros(n_words, dtype=np.uint32) if include_rc else None
    nm = np.zeros(n_bytes, dtype=np.uint8) if include_n_mask else None
    check(lib().bgo_encode_genome(raw.ctypes.data, ptr(lens), lens.size, int(device),
                                  fwd.ctypes.data if n_words else None,
                                  None if rc is None or not n_words else rc.ctypes.data,
                                  None if nm is None or not n_bytes else nm.ctypes.data),
          "bgo_encode_genome")
    return fwd, rc, nm


def probe_int_throughput(op, device=0):
    """Measured Gop/s of LOP3 (op 0), POPC (1) or 32-bit add (2)."""
    v = ctypes.c_double()
    check(tools_lib().bgo_probe_int_throughput(int(device), int(op), ctypes.byref(v)),
          "bgo_probe_int_throughput")
    return v.value


def library_path():
    return _build.LIB_PATH


def lib():
    """The loaded library; raises NativeLibraryMissing when it was not built."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not os.path.exists(path):
            raise NativeLibraryMissing(
                f"native library {path} is not built; run "
                "`python -c 'import beguidedoff_gb300.build as b; b.build()'` (needs nvcc)")
        L = ctypes.CDLL(path)
        for name, (args, res) in _SIGS.items():
            if name in TOOLS_EXPORTED:
                continue
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = L
    return _LIB


_TOOLS = None


def tools_lib():
    """The tools library (synthetic genomes, integer-pipe probe)."""
    global _TOOLS
    if _TOOLS is None:
        lib()
        path = _build.TOOLS_PATH
        if not os.path.exists(path):
            raise NativeLibraryMissing(f"tools library {path} is not built")
        L = ctypes.CDLL(path)
        for name in TOOLS_EXPORTED:
            args, res = _SIGS[name]
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _TOOLS = L
    return _TOOLS


def last_error():
    buf = ctypes.create_string_buffer(4096)
    lib().bgo_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc, where):
    if rc != BGO_OK:
        raise BgoError(rc, where, last_error())


def ptr(a):
    """Address of a contiguous numpy array (None for an empty one)."""
    if a is None or a.size == 0:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def device_count():
    n = ctypes.c_int(0)
    check(lib().bgo_device_count(ctypes.byref(n)), "bgo_device_count")
    return n.value


class HostBuffer:
    """Page-locked host memory viewed as a numpy array."""

    def __init__(self, shape, dtype):
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * dtype.itemsize
        p = ctypes.c_void_p()
        check(lib().bgo_host_alloc(ctypes.byref(p), max(n, 1)), "bgo_host_alloc")
        self._p = p
        buf = (ctypes.c_char * max(n, 1)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def close(self):
        if self._p is not None and self._p.value:
            self.array = None
            lib().bgo_host_free(self._p)
        self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Strand:
    """One strand array resident on the device (H/L/N bit planes)."""

    def __init__(self, packed, total_bp, n_mask_le=None, device=0, stream=None):
        packed = np.ascontiguousarray(packed, dtype=np.uint32)
        nm = None if n_mask_le is None else np.ascontiguousarray(n_mask_le, dtype=np.uint8)
        h = ctypes.c_void_p()
        check(lib().bgo_genome_create(ptr(packed), packed.size, int(total_bp), ptr(nm),
                                      0 if nm is None else nm.size, int(device), stream,
                                      ctypes.byref(h)), "bgo_genome_create")
        self.handle = h
        self.total_bp = int(total_bp)
        self.device = int(device)

    def upload(self, packed, n_mask_le=None, stream=None):
        """Replace the contents in place (same total_bp), queued on `stream`
        (bgo_genome_upload); the arrays must stay valid until the stream
        has run the copies."""
        packed = np.ascontiguousarray(packed, dtype=np.uint32)
        nm = None if n_mask_le is None else np.ascontiguousarray(n_mask_le, dtype=np.uint8)
        check(lib().bgo_genome_upload(self.handle, ptr(packed), packed.size, ptr(nm),
                                      0 if nm is None else nm.size, stream), "bgo_genome_upload")

    def info(self):
        tb, hn, nb = ctypes.c_int64(), ctypes.c_int(), ctypes.c_int64()
        check(lib().bgo_genome_info(self.handle, ctypes.byref(tb), ctypes.byref(hn),
                                    ctypes.byref(nb)), "bgo_genome_info")
        return {"total_bp": tb.value, "has_n_mask": bool(hn.value), "device_bytes": nb.value}

    def close(self):
        if self.handle is not None and self.handle.value:
            lib().bgo_genome_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Stream:
    """A non-blocking CUDA stream (bgo_stream_create); pass ``.handle`` as the
    stream argument."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        check(lib().bgo_stream_create(int(device), ctypes.byref(h)), "bgo_stream_create")
        self.handle = h

    def close(self):
        if self.handle is not None and self.handle.value:
            lib().bgo_stream_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Tuning(ctypes.Structure):
    """bgo_tuning: launch parameters of scan modes 2 and 3 (0 = default)."""
    _fields_ = [("chunk_sites", ctypes.c_int32), ("group_guides", ctypes.c_int32),
                ("ctas_per_sm", ctypes.c_int32), ("split_families", ctypes.c_int32),
                ("min_blocks", ctypes.c_int32), ("tolerance", ctypes.c_int32),
                ("family_form", ctypes.c_int32), ("inline_entries", ctypes.c_int32),
                ("range_walk", ctypes.c_int32), ("prefilter", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 2)]


class Plan:
    """Guide rows grouped into PAM families on the device."""

    def __init__(self, engine, guide_encoded, pam_masks, pam_lens, pam_3prime, stream=None):
        self.guides = np.ascontiguousarray(guide_encoded, dtype=np.uint64)
        n = self.guides.size
        pm = np.zeros((n, 6), dtype=np.uint8)
        if n:
            src = np.asarray(pam_masks, dtype=np.uint8).reshape(n, -1)
            pm[:, :min(6, src.shape[1])] = src[:, :6]
        self.pam_masks = pm
        self.pam_lens = np.ascontiguousarray(pam_lens, dtype=np.uint8)
        self.pam_3prime = np.ascontiguousarray(pam_3prime, dtype=np.uint8)
        h = ctypes.c_void_p()
        check(lib().bgo_plan_create(engine.handle, ptr(self.guides), ptr(self.pam_masks),
                                    ptr(self.pam_lens), ptr(self.pam_3prime), n, stream,
                                    ctypes.byref(h)), "bgo_plan_create")
        self.handle = h
        self.n_guides = n

    def info(self):
        nf, ng = ctypes.c_int32(), ctypes.c_int32()
        check(lib().bgo_plan_info(self.handle, ctypes.byref(nf), ctypes.byref(ng)),
              "bgo_plan_info")
        return {"n_families": nf.value, "n_guides": ng.value}

    def set_tuning(self, chunk_sites=0, group_guides=0, ctas_per_sm=0, split_families=0,
                   min_blocks=0, tolerance=0, inline_entries=0, range_walk=0, prefilter=0):
        """Launch parameters of scan modes 2 and 3 (see bgo_plan_set_tuning)."""
        t = Tuning(int(chunk_sites), int(group_guides), int(ctas_per_sm), int(split_families),
                   int(min_blocks), int(tolerance), 0, int(inline_entries), int(range_walk),
                   int(prefilter))
        check(lib().bgo_plan_set_tuning(self.handle, ctypes.byref(t)), "bgo_plan_set_tuning")
        self.tuning = {"chunk_sites": int(chunk_sites), "group_guides": int(group_guides),
                       "ctas_per_sm": int(ctas_per_sm), "split_families": int(split_families),
                       "min_blocks": int(min_blocks), "tolerance": int(tolerance),
                       "inline_entries": int(inline_entries), "range_walk": int(range_walk),
                       "prefilter": int(prefilter)}

    def set_family_tuning(self, family, chunk_sites=0, min_blocks=0, tolerance=0, form=0,
                          ctas_per_sm=0, inline_entries=0, range_walk=0, prefilter=0):
        """Launch parameters of one PAM family in split launches (form 0:
        segment index, 1: every guide compared)."""
        t = Tuning(int(chunk_sites), 0, int(ctas_per_sm), 1, int(min_blocks), int(tolerance),
                   int(form), int(inline_entries), int(range_walk), int(prefilter))
        check(lib().bgo_plan_set_family_tuning(self.handle, int(family), ctypes.byref(t)),
              "bgo_plan_set_family_tuning")

    def families(self):
        """Family index of each plan row (-1: the row never matches)."""
        out = np.empty(max(self.n_guides, 1), dtype=np.int32)
        check(lib().bgo_plan_families(self.handle, out.ctypes.data), "bgo_plan_families")
        return out[:self.n_guides]

    def close(self):
        if self.handle is not None and self.handle.value:
            lib().bgo_plan_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Engine:
    """Per-device scan workspace (hit buffer and counters)."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        check(lib().bgo_engine_create(int(device), ctypes.byref(h)), "bgo_engine_create")
        self.handle = h
        self.device = int(device)

    def launch(self, plan, strands, n_encoded, max_mismatches, mode=1, stream=None):
        arr = (ctypes.c_void_p * len(strands))(*[s.handle.value for s in strands])
        ne = np.ascontiguousarray(n_encoded, dtype=np.int32)
        check(lib().bgo_scan_launch(self.handle, plan.handle, arr, ptr(ne), len(strands),
                                    int(max_mismatches), int(mode), stream), "bgo_scan_launch")

    def collect(self, stream=None):
        """Waits for the last launch; returns (n_hits, sorted keys or None if
        the device buffer overflowed)."""
        n = ctypes.c_int64()
        check(lib().bgo_scan_collect(self.handle, None, 0, ctypes.byref(n), stream),
              "bgo_scan_collect")
        if n.value > self.info()["hit_capacity"]:
            return n.value, None
        keys = np.empty(n.value, dtype=np.uint64)
        if n.value == 0:
            return 0, keys
        check(lib().bgo_scan_collect(self.handle, ptr(keys), keys.size, ctypes.byref(n), stream),
              "bgo_scan_collect")
        return n.value, keys

    def scan_time(self, plan, strands, n_encoded, max_mismatches, mode, reps=2, stream=None):
        """Fastest of `reps` event-timed scans after one untimed launch (ms)."""
        arr = (ctypes.c_void_p * len(strands))(*[s.handle.value for s in strands])
        ne = np.ascontiguousarray(n_encoded, dtype=np.int32)
        ms = ctypes.c_double()
        check(lib().bgo_scan_time(self.handle, plan.handle, arr, ptr(ne), len(strands),
                                  int(max_mismatches), int(mode), int(reps), stream,
                                  ctypes.byref(ms)), "bgo_scan_time")
        return ms.value

    def hit_count(self, stream=None):
        n = ctypes.c_int64()
        check(lib().bgo_scan_collect(self.handle, None, 0, ctypes.byref(n), stream),
              "bgo_scan_collect")
        return n.value

    def pairs_evaluated(self, stream=None):
        """(PAM-passing position, guide) pairs counted by the last launch."""
        n = ctypes.c_int64()
        check(lib().bgo_scan_stats(self.handle, ctypes.byref(n), stream), "bgo_scan_stats")
        return n.value

    def reserve(self, n_hits):
        check(lib().bgo_engine_reserve(self.handle, int(n_hits)), "bgo_engine_reserve")

    def complete(self, plan, strands, n_encoded, max_mismatches, mode=1, stream=None):
        """After launch(): makes the hit buffer hold every hit of that scan
        (bgo_scan_complete: on overflow, grows it and rescans only the
        granules whose keys were dropped); returns the exact hit count."""
        arr = (ctypes.c_void_p * len(strands))(*[s.handle.value for s in strands])
        ne = np.ascontiguousarray(n_encoded, dtype=np.int32)
        n = ctypes.c_int64()
        check(lib().bgo_scan_complete(self.handle, plan.handle, arr, ptr(ne), len(strands),
                                      int(max_mismatches), int(mode), stream, ctypes.byref(n)),
              "bgo_scan_complete")
        return n.value

    def scan(self, plan, strands, n_encoded, max_mismatches, mode=1, stream=None):
        """Launch + complete + collect: every hit key, sorted."""
        self.launch(plan, strands, n_encoded, max_mismatches, mode, stream)
        self.complete(plan, strands, n_encoded, max_mismatches, mode, stream)
        n, keys = self.collect(stream)
        if keys is None:
            raise BgoError(BGO_ERR_STATE, "scan", "hit buffer overflow after completion")
        return keys

    def info(self):
        cap, nl = ctypes.c_int64(), ctypes.c_int64()
        check(lib().bgo_engine_info(self.handle, ctypes.byref(cap), ctypes.byref(nl)),
              "bgo_engine_info")
        return {"hit_capacity": cap.value, "launches": nl.value}

    def launch_count(self):
        return self.info()["launches"]

    def transfer(self):
        """Bytes copied by this engine's calls: {"h2d": ..., "d2h": ...}."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        check(lib().bgo_engine_transfer(self.handle, ctypes.byref(a), ctypes.byref(b)),
              "bgo_engine_transfer")
        return {"h2d": a.value, "d2h": b.value}

    # input rows per bgo_epilogue_run call: its scratch holds a 16 KB rank
    # histogram per row, so larger row sets run in chunks (rows are independent)
    EPILOGUE_ROWS_PER_CALL = 131072

    def epilogue(self, plan, strands, inputs, chrom_offsets, chrom_lengths, chrom_rank,
                 rank_table, n_top, stream=None):
        """Device epilogue of the last scan (bgo_epilogue_run + fetch):
        (below[n_inputs], group_counts[n_plan_rows, 2], row_counts[n_inputs],
        records grouped by input row)."""
        inputs = np.ascontiguousarray(inputs, dtype=INPUT_ROW_DTYPE)
        step = self.EPILOGUE_ROWS_PER_CALL
        if inputs.size > step:
            parts = [self.epilogue(plan, strands, inputs[i:i + step], chrom_offsets,
                                   chrom_lengths, chrom_rank, rank_table, n_top, stream)
                     for i in range(0, inputs.size, step)]
            recs = []
            for i, p in zip(range(0, inputs.size, step), parts):
                r = p[3].copy()
                r["input_row"] += i
                recs.append(r)
            return (np.concatenate([p[0] for p in parts]), parts[0][1],
                    np.concatenate([p[2] for p in parts]), np.concatenate(recs))
        offs = np.ascontiguousarray(chrom_offsets, dtype=np.int64)
        lens = np.ascontiguousarray(chrom_lengths, dtype=np.int64)
        crank = np.ascontiguousarray(chrom_rank, dtype=np.int32)
        rt = np.ascontiguousarray(rank_table, dtype=np.uint32)
        arr = (ctypes.c_void_p * len(strands))(*[s.handle.value for s in strands])
        below = np.zeros(max(inputs.size, 1), dtype=np.int64)
        counts = np.zeros(max(inputs.size, 1), dtype=np.int64)
        groups = np.zeros(max(2 * plan.n_guides, 2), dtype=np.int64)
        n = ctypes.c_int64()
        check(lib().bgo_epilogue_run(
            self.handle, plan.handle, arr, len(strands), ptr(inputs), inputs.size, ptr(offs),
            ptr(lens), ptr(crank), offs.size, ptr(rt), int(n_top), below.ctypes.data,
            groups.ctypes.data, counts.ctypes.data, ctypes.byref(n), stream), "bgo_epilogue_run")
        recs = np.zeros(n.value, dtype=RECORD_DTYPE)
        check(lib().bgo_epilogue_fetch(self.handle, recs.ctypes.data if n.value else None,
                                       n.value, stream), "bgo_epilogue_fetch")
        return (below[:inputs.size], groups[:2 * plan.n_guides].reshape(-1, 2),
                counts[:inputs.size], recs)

    def close(self):
        if self.handle is not None and self.handle.value:
            lib().bgo_engine_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Graph:
    """A scan captured once into a CUDA graph; replay() rescans (keep the
    engine, plan and strands alive and do not reserve the engine meanwhile)."""

    def __init__(self, engine, plan, strands, n_encoded, max_mismatches, mode=2):
        arr = (ctypes.c_void_p * len(strands))(*[s.handle.value for s in strands])
        ne = np.ascontiguousarray(n_encoded, dtype=np.int32)
        h = ctypes.c_void_p()
        check(lib().bgo_graph_create(engine.handle, plan.handle, arr, ptr(ne), len(strands),
                                     int(max_mismatches), int(mode), ctypes.byref(h)),
              "bgo_graph_create")
        self.handle = h
        self._keep = (engine, plan, strands)

    def replay(self, stream=None):
        check(lib().bgo_graph_launch(self.handle, stream), "bgo_graph_launch")

    def close(self):
        if self.handle is not None and self.handle.value:
            lib().bgo_graph_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def split_keys(keys):
    """(row, strand_slot, position, mismatches) int64 arrays from hit keys."""
    keys = np.asarray(keys, dtype=np.uint64)
    return ((keys >> np.uint64(39)).astype(np.int64),
            ((keys >> np.uint64(38)) & np.uint64(1)).astype(np.int64),
            ((keys >> np.uint64(6)) & np.uint64(0xFFFFFFFF)).astype(np.int64),
            (keys & np.uint64(63)).astype(np.int64))
