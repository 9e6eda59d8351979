"""Member partitioning for multi-GPU ensembles, exercised with gloo ranks on the CPU."""
import os

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from pyprop_gb300.ensemble import partition_members


@pytest.mark.parametrize("n,world", [(256, 2), (7, 3), (3, 4), (0, 2)])
def test_partition_covers_every_member_once(n, world):
    seen = []
    for r in range(world):
        a, b = partition_members(n, world, r)
        assert 0 <= a <= b <= n
        seen.extend(range(a, b))
    assert seen == list(range(n))
    sizes = [partition_members(n, world, r)[1] - partition_members(n, world, r)[0] for r in range(world)]
    assert max(sizes) - min(sizes) <= 1


def _worker(rank, world, port, n, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    a, b = partition_members(n, world, rank)
    # each rank "advances" its members: the job total is the sum of member steps, no data exchange
    steps = torch.tensor([float(b - a)])
    dist.all_reduce(steps)
    t = torch.tensor([0.1 * (rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)  # the job time is the slowest rank's
    if rank == 0:
        q.put((steps.item(), t.item()))
    dist.destroy_process_group()


def test_gloo_two_ranks_replica_accounting():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29731
    procs = [ctx.Process(target=_worker, args=(r, 2, port, 256, q)) for r in range(2)]
    for p in procs:
        p.start()
    steps, t = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
    assert steps == 256.0 and abs(t - 0.2) < 1e-6
