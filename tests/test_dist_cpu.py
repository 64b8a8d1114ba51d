"""Replicas-only multi-GPU plumbing of bench.py, exercised with 2 gloo ranks on CPU:
each rank times its own solve, the job time is the max over ranks and the value counts
every rank's steps."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    d = bench.Dist(world, backend="gloo")  # CPU ranks, also where a GPU is visible
    d.barrier()
    my_ms = 100.0 + 50.0 * rank          # rank 1 is the slow one
    mx = d.max(my_ms)
    q.put((rank, mx, bench.aggregate(d.world, 40, mx)))
    d.close()


def test_two_rank_replica_aggregation():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, val in res:
        assert mx == 150.0
        assert val == pytest.approx(2 * 40 / 0.150)
