"""Replicas across ranks (the multi-GPU form of the path: independent simulations, no
exchange): the bench's aggregation over a world of 2 gloo ranks on the CPU -- the job's
time is the slowest rank's, its work the sum of the ranks'."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t, cu = bench.reduce_replicas(1.0 + rank, 1000.0 * (rank + 1), dist, "cpu")
    out.put((rank, t, cu))
    dist.barrier()
    dist.destroy_process_group()


def test_reduce_replicas_gloo_world2():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2.0, 3000.0), (1, 2.0, 3000.0)]


def test_reduce_replicas_single():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_replicas(1.5, 42, None) == (1.5, 42.0)
