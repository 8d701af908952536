"""The bench's multi-rank path on CPU: two gloo ranks, max-over-ranks timing,
barrier, whole-job throughput of replicas, and a reference arm that runs on
rank 0 only."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update({"WORLD_SIZE": str(ws), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    w, r, _ = bench.dist_setup("gloo")
    assert (w, r) == (ws, rank)
    bench.barrier(w)
    t = bench.dist_max(1.0 + rank, w)          # rank 1 is the slow one
    out.put((rank, t, bench.replica_value(w, 100.0, t)))
    bench.barrier(w)
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.0, 2.0]
    assert all(abs(r[2] - 100.0) < 1e-9 for r in res)   # 2 ranks x 100 units / 2 s


def test_reference_arm_prints_on_rank_zero_only(capsys, monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        pass

    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.bench_reference(Args(), 2, 1) is None   # rank 1 does no work
    assert capsys.readouterr().out == ""
