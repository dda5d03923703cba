"""Replicas on several processes (gloo, CPU): every rank takes a disjoint
contiguous range of scenes, the union is the whole batch, and the per-rank
work is balanced.  The data path needs no collective; only this bookkeeping
is exchanged."""
import os

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from fledge_gb300.shard import partition_scenes


def _worker(rank, world, port, counts, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import torch
    ranges = partition_scenes(counts, world)
    a, b = ranges[rank]
    mine = torch.tensor([a, b, int(sum(counts[a:b]))], dtype=torch.int64)
    out = [torch.zeros(3, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(out, mine)
    if rank == 0:
        q.put([o.tolist() for o in out])
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_partition_over_gloo(world):
    counts = np.round(np.exp(np.random.default_rng(0).uniform(np.log(1e3), np.log(1e6), 256))).astype(int).tolist()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + world + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, world, port, counts, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    covered = []
    for a, b, w in got:
        covered += list(range(a, b))
    assert covered == list(range(256))
    works = [w for _, _, w in got]
    # each cumulative cut lands within half a scene of its target
    assert max(works) - min(works) <= 2 * max(counts)


def test_partition_edge_cases():
    assert partition_scenes([5], 1) == [(0, 1)]
    r = partition_scenes([1, 1, 1, 1], 4)
    assert r == [(0, 1), (1, 2), (2, 3), (3, 4)]
    r = partition_scenes([100, 1, 1, 1], 2)
    assert r[0] == (0, 1) and r[1] == (1, 4)
