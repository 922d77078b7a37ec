"""bench.py's multi-process helpers on CPU: two gloo ranks (the replicas
mode of `bench.py --gpus N`: per-rank timings, max over ranks, barriers)."""
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


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w, loc = bench.dist_env()
    dist = bench.init_dist(w)
    bench.barrier(dist)
    m = bench.max_over_ranks(dist, 1.5 + r)  # rank r "took" 1.5 + r seconds
    bench.barrier(dist)
    out.put((r, w, loc, m))
    dist.destroy_process_group()


def test_two_gloo_ranks_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert res == [(0, 2, 0, 2.5), (1, 2, 1, 2.5)]


def test_single_process_needs_no_process_group(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench.dist_env() == (0, 1, 0)
    assert bench.init_dist(1) is None
    assert bench.max_over_ranks(None, 3.0) == 3.0
