"""Sharding of the batched-droplet workload over ranks (no data-path collective): two gloo ranks on
the CPU each take their share, and the only exchange, a final metrics reduction, shows that the
shares cover every droplet exactly once with balanced particle counts."""
import os

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from fjsph_gb300 import cases


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import torch
    b = cases.droplet_batch(n_drops=40, n_min=200, n_max=3000, seed=9)
    ids = cases.shard_ids(len(b.counts), b.counts, rank, world)
    sub = b.subset(ids)
    # the shard is a batch of its own: same particles as the selected droplets of the full batch
    for k, g in enumerate(ids):
        np.testing.assert_array_equal(sub.case.state.xi[sub.first[k]:sub.first[k + 1]],
                                      b.case.state.xi[b.first[g]:b.first[g + 1]])
    mask = torch.zeros(len(b.counts), dtype=torch.int64)
    mask[torch.as_tensor(ids)] = 1
    n = torch.tensor([sub.case.state.n], dtype=torch.int64)
    nmax = n.clone()
    dist.all_reduce(mask)
    dist.all_reduce(n)
    dist.all_reduce(nmax, op=dist.ReduceOp.MAX)
    if rank == 0:
        q.put((mask.tolist(), int(n), int(nmax), int(b.case.state.n)))
    dist.destroy_process_group()


def test_shards_cover_every_droplet_once():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    mask, n, nmax, total = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert mask == [1] * 40
    assert n == total
    assert nmax <= 0.55 * total  # balanced within 10 %


@pytest.mark.parametrize("world", [1, 3, 8])
def test_shard_ids_partition(world):
    b = cases.droplet_batch(n_drops=50, n_min=200, n_max=3000, seed=3)
    parts = [cases.shard_ids(50, b.counts, r, world) for r in range(world)]
    allids = np.sort(np.concatenate(parts))
    np.testing.assert_array_equal(allids, np.arange(50))
