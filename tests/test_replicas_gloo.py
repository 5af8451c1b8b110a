"""The N > 1 path of bench.py on CPU: each rank is an independent replica, the job time is the
maximum over ranks and the units add up.  Two gloo ranks, no GPU."""
from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank: int, world: int, port: int, q):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    t, u = bench.aggregate(10.0 + 5.0 * rank, 1000.0 * (rank + 1), world, None)
    q.put((rank, t, u))
    dist.destroy_process_group()


def test_two_replicas_max_time_sum_units():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for _, t, u in res:
        assert t == pytest.approx(15.0)
        assert u == pytest.approx(3000.0)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.aggregate(3.0, 7.0, 1) == (3.0, 7.0)
