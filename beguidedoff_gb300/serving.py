"""Continuous-batching search service over a genome resident in HBM.

The reference answers one ``search()`` call at a time (beguidedoff/finder.py
:475-679), scanning the genome once per call.  A service with many small
requests wastes most of each scan, so here requests are queued and batched:

* The genome is uploaded once (the finder's strands) and stays resident.
* ``n_slots`` workers each own an engine (hit buffer and epilogue scratch)
  and a non-blocking CUDA stream.  A worker that becomes free takes the next
  batch at once, so requests that arrive while other batches are on the GPU
  are admitted as soon as a slot and memory allow.  Their work then overlaps
  with the running batches: scans on separate streams, and host assembly of
  one batch beside the device work of another.
* A batch holds queued requests with one max_mismatches value, in arrival
  order, up to ``max_batch_guides`` guides.  Each request is admitted by its
  output-buffer memory: the expected hit keys (guides x a per-K hits-per-guide
  estimate that follows what finished batches produced) plus the epilogue's
  per-input-row scratch.  The sum over in-flight batches stays within
  ``memory_bytes``; a request that is larger than the whole budget runs alone.
* One plan, scan and device epilogue serve the whole batch.  Input rows,
  options (return_all, threshold) and assembly stay per request, so every
  request gets the table ``search()`` would give it alone.

``Batcher`` is the admission and batching policy with no GPU in it;
``SearchServer`` runs it on the device.
"""
import threading
import time
from collections import deque
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import Dict, List, Optional

from . import _native
from .finder import beguidedoff
from .types import GuideInput

# epilogue scratch per input row: the 4,096-bin rank histogram and row state
EPILOGUE_BYTES_PER_ROW = 4096 * 4 + 128
KEY_BYTES = 8
# starting hits-per-guide estimates per max_mismatches (a 3.1 Gbp genome,
# mixed PAM families); replaced by what finished batches produce
PRIOR_HITS_PER_GUIDE = {0: 4, 1: 8, 2: 30, 3: 200, 4: 1500, 5: 9000, 6: 40000, 7: 150000}


@dataclass
class Request:
    guides: List[GuideInput]
    max_mismatches: int
    return_all: bool = False
    count_score_threshold: Optional[float] = None
    rid: int = 0
    est_bytes: int = 0
    t_submit: float = 0.0
    t_start: float = 0.0
    t_done: float = 0.0
    batch: int = -1
    future: Future = field(default_factory=Future)


class Batcher:
    """FIFO admission by output-buffer memory and batching by max_mismatches
    (thread-safe; no GPU)."""

    def __init__(self, memory_bytes: int, max_batch_guides: int = 2048,
                 prior: Optional[Dict[int, float]] = None):
        self.memory_bytes = int(memory_bytes)
        self.max_batch_guides = int(max_batch_guides)
        self.hits_per_guide = dict(PRIOR_HITS_PER_GUIDE if prior is None else prior)
        self.queue: deque = deque()
        self.in_flight = 0
        self.cv = threading.Condition()
        self.closed = False
        self.n_batches = 0

    def estimate(self, req: Request) -> int:
        hpg = self.hits_per_guide.get(req.max_mismatches, 200000)
        return int(len(req.guides) * (hpg * KEY_BYTES + EPILOGUE_BYTES_PER_ROW))

    def add(self, req: Request) -> None:
        with self.cv:
            if self.closed:
                raise RuntimeError("server is closed")
            req.est_bytes = self.estimate(req)
            self.queue.append(req)
            self.cv.notify_all()

    def take(self, timeout: Optional[float] = None) -> List[Request]:
        """Blocks until a batch can be admitted; [] when closed and drained
        (or on timeout).  The batch starts with the oldest queued request and
        adds later ones with the same max_mismatches while guides and memory
        allow."""
        with self.cv:
            deadline = None if timeout is None else time.monotonic() + timeout
            while True:
                batch = self._form()
                if batch:
                    self.n_batches += 1
                    for r in batch:
                        r.batch = self.n_batches
                    return batch
                if self.closed and not self.queue:
                    return []
                wait = None if deadline is None else deadline - time.monotonic()
                if wait is not None and wait <= 0:
                    return []
                self.cv.wait(wait)

    def _form(self) -> List[Request]:
        if not self.queue:
            return []
        first = self.queue[0]
        free = self.memory_bytes - self.in_flight
        if first.est_bytes > free and self.in_flight > 0:
            return []  # wait for memory (FIFO: nothing may overtake the head)
        batch, guides, used = [], 0, 0
        for r in list(self.queue):
            if r.max_mismatches != first.max_mismatches:
                continue
            if batch and (guides + len(r.guides) > self.max_batch_guides or
                          used + r.est_bytes > free):
                break
            batch.append(r)
            guides += len(r.guides)
            used += r.est_bytes
        for r in batch:
            self.queue.remove(r)
        self.in_flight += used
        return batch

    def release(self, batch: List[Request], hits: Optional[int] = None) -> None:
        with self.cv:
            self.in_flight -= sum(r.est_bytes for r in batch)
            n_guides = sum(len(r.guides) for r in batch)
            if hits is not None and n_guides:
                k = batch[0].max_mismatches
                old = self.hits_per_guide.get(k, hits / n_guides)
                self.hits_per_guide[k] = 0.5 * old + 0.5 * max(1.0, hits / n_guides)
            self.cv.notify_all()

    def close(self) -> None:
        with self.cv:
            self.closed = True
            self.cv.notify_all()


class SearchServer:
    """Continuous-batching extensive-mode search over a resident genome.

    ``submit()`` returns a Future whose result is the table ``search()``
    returns for the same guides and options.
    """

    def __init__(self, genome_path: Optional[str] = None, genome_data: Optional[dict] = None,
                 device: Optional[str] = None, n_slots: int = 2, memory_bytes: int = 8 << 30,
                 max_batch_guides: int = 2048, n_top_offtargets: int = 3,
                 results_per_guide: int = 10240, max_results_per_guide: Optional[int] = None,
                 scan_mode="auto", tune_per_k: bool = True):
        self.finder = beguidedoff(genome_path, max_mismatches=4, device=device,
                                  n_top_offtargets=n_top_offtargets,
                                  results_per_guide=results_per_guide,
                                  max_results_per_guide=max_results_per_guide,
                                  genome_data=genome_data, scan_mode=scan_mode)
        # batches mix PAM families and sizes freely: one autotuner choice per
        # max_mismatches instead of one per plan signature
        self.finder.tune_per_k = tune_per_k
        dev = self.finder.device_index
        self.batcher = Batcher(memory_bytes, max_batch_guides)
        self.slots = [(_native.Engine(dev), _native.Stream(dev)) for _ in range(n_slots)]
        self._rid = 0
        self._lock = threading.Lock()
        self.done: List[Request] = []
        self.batches: List[dict] = []
        self._workers = [threading.Thread(target=self._work, args=(i,), daemon=True)
                         for i in range(n_slots)]
        for w in self._workers:
            w.start()

    def warmup(self, max_mismatches=(3, 4, 5), pams=("NGG", "NG", "NNGRRT", "NNNRRT", "NRN"),
               sizes=(8, 48, 200, 800, 1600), seed: int = 0) -> dict:
        """Runs the autotuner for every (max_mismatches, size class) on random
        guides cycling through `pams`, so that no request pays for tuning."""
        import numpy as np

        rng = np.random.default_rng(seed)
        f = self.finder
        if f.scan_mode != "auto":
            return {}
        out = {}
        for k in max_mismatches:
            for n in sizes:
                seqs = ["".join(rng.choice(list("ACGT"), 20)) for _ in range(n)]
                plan_pams = [pams[i % len(pams)] for i in range(n)]
                plan = f._plan(seqs, plan_pams)
                try:
                    f._mode_for(plan, plan_pams, k)
                    out[(k, n)] = f.last_choice.name
                finally:
                    plan.close()
        return out

    def submit(self, guides: List[GuideInput], max_mismatches: int = 4, return_all: bool = False,
               count_score_threshold: Optional[float] = None) -> Future:
        with self._lock:
            self._rid += 1
            rid = self._rid
        req = Request(list(guides), int(max_mismatches), return_all, count_score_threshold, rid,
                      t_submit=time.perf_counter())
        self.batcher.add(req)
        return req.future

    def _work(self, slot: int) -> None:
        engine, stream = self.slots[slot]
        f = self.finder
        while True:
            batch = self.batcher.take()
            if not batch:
                return
            t0 = time.perf_counter()
            for r in batch:
                r.t_start = t0
            ready, reqs = [], []
            for r in batch:
                try:
                    keys, mapping = f._prepare(r.guides)
                except Exception as exc:
                    self._finish(r, exc)
                    continue
                ready.append(r)
                reqs.append({"keys": keys, "mapping": mapping, "guides": r.guides,
                             "return_all": r.return_all,
                             "count_score_threshold": r.count_score_threshold})
            hits = None
            times: dict = {}
            try:
                if reqs:
                    info: dict = {}
                    results = f._run_batch(reqs, batch[0].max_mismatches, engine,
                                           stream.handle, info=info)
                    hits = info.get("hits")
                    times = {k: info[k] for k in ("plan_s", "scan_s", "epilogue_s",
                                                  "assemble_s") if k in info}
                    for r, res in zip(ready, results):
                        self._finish(r, res)
            except Exception as exc:
                for r in ready:
                    if not r.future.done():
                        self._finish(r, exc)
            finally:
                self.batcher.release(batch, hits)
                with self._lock:
                    self.batches.append({"slot": slot, "requests": len(batch),
                                         "guides": sum(len(r.guides) for r in batch),
                                         "k": batch[0].max_mismatches, "hits": hits,
                                         "seconds": time.perf_counter() - t0, **times})

    def _finish(self, r: Request, res) -> None:
        r.t_done = time.perf_counter()
        with self._lock:
            self.done.append(r)
        if isinstance(res, Exception):
            r.future.set_exception(res)
        else:
            r.future.set_result(res)

    def latencies(self) -> List[float]:
        with self._lock:
            return [r.t_done - r.t_submit for r in self.done]

    def close(self) -> None:
        self.batcher.close()
        for w in self._workers:
            w.join()
        for e, s in self.slots:
            e.close()
            s.close()
        self.slots = []
        self.finder.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
