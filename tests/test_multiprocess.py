"""Replica logic of bench.py with two gloo ranks on CPU: every rank times
its own simulation, the job time is the max over ranks and the throughput
counts all ranks' points."""

import os
import socket

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import sys

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    dist = bench.dist_init("gloo")
    my_secs = 1.0 + rank  # rank 1 is the slow one
    bench.barrier(dist)
    m = bench.reduce_max(my_secs, dist, device="cpu")
    v = bench.aggregate_throughput(1000, 10, world, m)
    q.put((rank, m, v))
    dist.destroy_process_group()


def test_two_rank_max_and_aggregate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, m, v in out:
        assert m == 2.0
        assert abs(v - 2 * 1000 * 10 / 2.0 / 1e6) < 1e-15
