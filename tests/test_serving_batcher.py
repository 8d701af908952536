"""Admission and batching policy of the serving loop (CPU, no GPU)."""
import threading
import time

from beguidedoff_gb300.serving import Batcher, Request
from beguidedoff_gb300.types import GuideInput


def _req(n, k, rid):
    g = [GuideInput(f"r{rid}_{i}", "A" * 20, "NGG", "3prime", 4, 8, "ABE") for i in range(n)]
    return Request(g, k, rid=rid)


def test_batches_group_by_k_in_arrival_order():
    b = Batcher(memory_bytes=1 << 40, max_batch_guides=100, prior={3: 1, 4: 1})
    for rid, (n, k) in enumerate([(10, 4), (5, 3), (20, 4), (90, 4), (7, 3)]):
        b.add(_req(n, k, rid))
    first = b.take(0)
    assert [r.rid for r in first] == [0, 2]          # 10 + 20, then 90 would exceed 100
    second = b.take(0)
    assert [r.rid for r in second] == [1, 4]         # the K=3 requests
    third = b.take(0)
    assert [r.rid for r in third] == [3]
    assert b.take(0) == []


def test_admission_by_output_memory():
    b = Batcher(memory_bytes=10_000_000, max_batch_guides=10_000, prior={5: 1000})
    per_guide = 1000 * 8 + 4096 * 4 + 128
    n = 10_000_000 // per_guide          # guides that fit the budget
    b.add(_req(n - 10, 5, 1))
    b.add(_req(20, 5, 2))
    a = b.take(0)
    assert [r.rid for r in a] == [1]     # the second does not fit beside it
    assert b.take(0) == []               # and waits for memory (nothing may overtake)
    b.release(a, hits=(n - 10) * 10)
    c = b.take(0)
    assert [r.rid for r in c] == [2]
    # the estimate follows observed hits
    assert b.hits_per_guide[5] < 1000


def test_oversized_request_runs_alone_and_close_drains():
    b = Batcher(memory_bytes=1000, max_batch_guides=10)
    b.add(_req(5, 4, 1))
    got = b.take(0)
    assert [r.rid for r in got] == [1]
    out = []

    def worker():
        while True:
            x = b.take()
            if not x:
                return
            out.append([r.rid for r in x])
            b.release(x)

    t = threading.Thread(target=worker)
    t.start()
    b.add(_req(1, 4, 2))
    time.sleep(0.05)
    assert out == []                      # waiting on memory held by request 1
    b.release(got)
    time.sleep(0.05)
    b.close()
    t.join(2)
    assert out == [[2]] and not t.is_alive()
