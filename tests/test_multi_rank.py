"""The N > 1 replica path of bench.py on CPU: two gloo ranks set up the
process group from the torchrun environment, meet at the barrier, and agree
on the max of their times and the sum of their paths (the bench's `value` is
sum(paths) / max(time)). The path shards by pixel with no data exchange, so
these reductions are the only collectives."""
from __future__ import annotations

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank: int, world: int, port: int, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench

    w, r, local, pg = bench.dist_setup(world)
    bench.barrier(pg)
    t = bench.max_over_ranks(pg, 1.5 + rank)      # per-rank device time
    p = bench.sum_over_ranks(pg, 1000.0 * (rank + 1))  # per-rank paths
    q.put((r, w, local, t, p))
    pg.destroy_process_group()


def test_two_gloo_ranks_reduce_like_the_bench():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    assert [o[0] for o in out] == [0, 1]
    for rank, world, local, t, paths in out:
        assert world == 2 and local == rank
        assert t == 2.5          # max over ranks
        assert paths == 3000.0   # sum over ranks


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    env = {k: os.environ.pop(k, None) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    try:
        w, r, local, pg = bench.dist_setup(1)
        assert (w, r, local, pg) == (1, 0, 0, None)
        assert bench.max_over_ranks(pg, 3.0) == 3.0 and bench.sum_over_ranks(pg, 4.0) == 4.0
    finally:
        for k, v in env.items():
            if v is not None:
                os.environ[k] = v
