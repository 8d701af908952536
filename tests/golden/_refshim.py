"""Test-only stand-ins that let the reference package run on a CPU-only host.

The reference extensive path needs numba (CUDA JIT), pandas, pysam and a CUDA
device. None of those exist in the build container, so this module installs
minimal stand-ins into ``sys.modules`` *before* the reference is imported:

* ``numba``: ``cuda.jit`` returns the Python function unchanged for device
  functions; a kernel becomes an object whose ``[grid, block]`` launch runs the
  kernel body literally, once per genome position, with ``blockDim.x == 1`` so
  the cooperative shared-memory load and ``syncthreads`` are trivially correct
  (beguidedoff/cuda_search.py:196-213).  ``atomic.add`` and ``popc`` are exact
  integer emulations; atomic order therefore equals genome order.
* ``pandas``: a row-list ``DataFrame`` with ``concat``, ``to_csv``, ``empty``.
* ``pysam``: ``FastaFile`` that parses a plain FASTA (for ``convert``).
* ``torch`` (inside the finder module only): reports a CUDA device so the
  finder's device check passes; tensors are never used by the kernel.

This file is used only by ``make_golden.py`` to record reference outputs; it is
never imported by the product or by the tests that run on the GPU machine.  The
reference checkout is found through the ``BGO_REFERENCE_ROOT`` environment
variable (``make_golden.py --reference DIR`` sets it).

``set_workers(n)`` makes a kernel launch run its blocks in ``n`` forked worker
processes, each over a contiguous block range with its own zeroed hit
counters; the parent appends the workers' hits in block order after the hits
already recorded, which is exactly the sequential run's atomic order (genome
order), with the same per-guide cap and exact counts.
"""
import multiprocessing
import os
import sys
import types

import numpy as np

REFERENCE_ROOT = os.environ.get("BGO_REFERENCE_ROOT", "")
_WORKERS = 1


def set_workers(n):
    global _WORKERS
    _WORKERS = max(1, int(n))


# ----------------------------------------------------------------------------
# numba stand-in
# ----------------------------------------------------------------------------
class _Dim:
    x = 0


class _DevArray(np.ndarray):
    def copy_to_host(self):
        return np.array(self, copy=True)


class _Kernel:
    def __init__(self, fn):
        self.fn = fn

    def __getitem__(self, cfg):
        grid, block = cfg

        def run(args, lo, hi):
            cuda = _cuda
            cuda.blockDim.x = 1
            cuda.threadIdx.x = 0
            for b in range(lo, hi):
                cuda.blockIdx.x = b
                self.fn(*args)

        def launch(*args):
            total = int(grid) * int(block)
            if _WORKERS == 1 or total < 4 * _WORKERS:
                run(args, 0, total)
                return
            # the search kernel's last three arguments are its outputs: per-guide
            # counters, positions and mismatches (beguidedoff/cuda_search.py:177-180)
            counts, hpos, hmm = args[-3], args[-2], args[-1]
            rpg = hpos.shape[1]
            bounds = np.linspace(0, total, _WORKERS + 1).astype(np.int64)
            # the workers are forked after this, so they inherit the kernel and
            # its arguments without pickling them
            _ACTIVE["fn"], _ACTIVE["args"] = self.fn, args
            ctx = multiprocessing.get_context("fork")
            with ctx.Pool(_WORKERS) as pool:
                parts = pool.starmap(_worker_run, [(int(bounds[w]), int(bounds[w + 1]))
                                                   for w in range(_WORKERS)])
            _ACTIVE.clear()
            for lc, lp, lm in parts:
                for g in range(counts.shape[0]):
                    k, c0 = int(lc[g]), int(counts[g])
                    keep = max(0, min(k, rpg - c0))
                    if keep:
                        hpos[g, c0:c0 + keep] = lp[g, :keep]
                        hmm[g, c0:c0 + keep] = lm[g, :keep]
                    counts[g] = c0 + k

        return launch


def _jit(fn=None, device=False, **_kw):
    if fn is None:
        return lambda f: _jit(f, device=device)
    if device:
        return fn
    return _Kernel(fn)


class _Shared:
    @staticmethod
    def array(n, dtype):
        return np.zeros(n, dtype=dtype)


class _Atomic:
    @staticmethod
    def add(arr, idx, val):
        old = int(arr[idx])
        arr[idx] = old + int(val)
        return old


_ACTIVE = {}


def _worker_run(lo, hi):
    """Blocks [lo, hi) of the active launch with fresh outputs; returns
    (counts, positions, mismatches)."""
    fn, args = _ACTIVE["fn"], _ACTIVE["args"]
    counts, hpos, hmm = args[-3], args[-2], args[-1]
    lc = np.zeros_like(counts)
    lp = np.zeros_like(hpos)
    lm = np.zeros_like(hmm)
    local = tuple(args[:-3]) + (lc, lp, lm)
    _cuda.blockDim.x = 1
    _cuda.threadIdx.x = 0
    for b in range(lo, hi):
        _cuda.blockIdx.x = b
        fn(*local)
    return lc, lp, lm


_cuda = types.SimpleNamespace(
    jit=_jit,
    threadIdx=_Dim(),
    blockIdx=_Dim(),
    blockDim=_Dim(),
    shared=_Shared,
    atomic=_Atomic,
    syncthreads=lambda: None,
    synchronize=lambda: None,
    popc=lambda v: int(v).bit_count(),
    to_device=lambda a: np.array(a, copy=True).view(_DevArray),
)
# three separate dim objects (threadIdx, blockIdx, blockDim)
_cuda.threadIdx = type("TI", (), {"x": 0})()
_cuda.blockIdx = type("BI", (), {"x": 0})()
_cuda.blockDim = type("BD", (), {"x": 1})()


def _make_numba():
    m = types.ModuleType("numba")
    m.cuda = _cuda
    m.uint32 = np.uint32
    m.uint64 = np.uint64
    m.int32 = np.int32
    m.int8 = np.int8
    m.uint8 = np.uint8
    return m


# ----------------------------------------------------------------------------
# pandas stand-in
# ----------------------------------------------------------------------------
class _DataFrame:
    def __init__(self, rows=None):
        self.rows = list(rows or [])

    def __len__(self):
        return len(self.rows)

    @property
    def empty(self):
        return not self.rows

    def to_csv(self, path, sep="\t", index=False):
        cols = list(self.rows[0].keys()) if self.rows else []
        with open(path, "w") as fh:
            fh.write(sep.join(cols) + "\n")
            for r in self.rows:
                fh.write(sep.join(str(r[c]) for c in cols) + "\n")


def _concat(dfs, ignore_index=True):
    out = _DataFrame()
    for d in dfs:
        out.rows.extend(d.rows)
    return out


def _make_pandas():
    m = types.ModuleType("pandas")
    m.DataFrame = _DataFrame
    m.concat = _concat
    m.notna = lambda v: v is not None and v == v
    return m


# ----------------------------------------------------------------------------
# pysam stand-in
# ----------------------------------------------------------------------------
class _FastaFile:
    def __init__(self, path):
        self._seqs = {}
        self.references = []
        name = None
        chunks = []
        with open(path) as fh:
            for line in fh:
                line = line.rstrip("\n")
                if line.startswith(">"):
                    if name is not None:
                        self._seqs[name] = "".join(chunks)
                    name = line[1:].split()[0]
                    self.references.append(name)
                    chunks = []
                elif line:
                    chunks.append(line)
        if name is not None:
            self._seqs[name] = "".join(chunks)

    def fetch(self, chrom, start=None, end=None):
        s = self._seqs[chrom]
        if start is None:
            return s
        return s[start:end]


def _make_pysam():
    m = types.ModuleType("pysam")
    m.FastaFile = _FastaFile
    return m


# ----------------------------------------------------------------------------
# torch stand-in for the finder module's device bookkeeping
# ----------------------------------------------------------------------------
class _FakeTensor:
    def __init__(self, a):
        self.a = a

    def to(self, _dev):
        return self


class _FakeDevice:
    def __init__(self, spec):
        self.type = str(spec).split(":")[0]

    def __str__(self):
        return self.type


_fake_torch = types.SimpleNamespace(
    device=_FakeDevice,
    cuda=types.SimpleNamespace(is_available=lambda: True),
    from_numpy=_FakeTensor,
)


def install():
    """Install the stand-ins and import the reference package.

    Returns the tuple (beguidedoff package, finder module, cuda_search module,
    genome_converter module).
    """
    if not REFERENCE_ROOT or not os.path.isdir(os.path.join(REFERENCE_ROOT, "beguidedoff")):
        raise SystemExit("set BGO_REFERENCE_ROOT (or make_golden.py --reference) to the "
                         "reference checkout")
    sys.dont_write_bytecode = True
    sys.modules.setdefault("numba", _make_numba())
    sys.modules.setdefault("pandas", _make_pandas())
    sys.modules.setdefault("pysam", _make_pysam())
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    import beguidedoff  # noqa: F401
    from beguidedoff import finder, cuda_search, genome_converter

    finder.torch = _fake_torch
    return beguidedoff, finder, cuda_search, genome_converter
