"""The benchmark's multi-rank timing on two gloo ranks (CPU): every rank waits at the barrier and
the reported time is the maximum over ranks, as `bench.py` takes it under torchrun."""
import os

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    bench.barrier(world)
    got = bench.reduce_max(world, 10.0 + 5.0 * rank)  # rank 1 is the slow one
    assert bench.reduce_max(1, 3.0) == 3.0  # one rank: no exchange
    q.put((rank, got))
    bench.barrier(world)
    dist.destroy_process_group()


def test_reduce_max_over_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29651
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 15.0), (1, 15.0)]
