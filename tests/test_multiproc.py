"""Member partitioning for multi-GPU ensembles, exercised with gloo ranks on the CPU.

Ensembles are replicas only: each rank advances its own contiguous share of the members
(``partition_members``) with no data-path collective; after the timed steps the ranks combine
the job throughput (member steps summed, the slowest rank's time) and gather the per-member
statistics into the ensemble's order. The tests run that host logic on two gloo ranks."""
import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from pyprop_gb300.ensemble import gather_member_values, hydrogen_ensemble_params, job_throughput, partition_members


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


def _member_size(prm):
    """Coefficients of a member's wavefunction: (lmax + 1) x B-splines."""
    return (prm["lmax"] + 1) * prm["nbsplines"]


def _worker(rank, world, port, n, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        a, b = partition_members(n, world, rank)
        params = hydrogen_ensemble_params(n)[a:b]   # this rank's members only
        steps = 5
        local = [_member_size(p) for p in params]    # a per-member statistic of this rank's members
        seconds = 0.1 * (rank + 1)                   # the ranks' own timed regions differ
        rate, units, secs = job_throughput(steps * len(params), seconds, world)
        gathered = gather_member_values(local, n, world, rank)
        if rank == 0:
            q.put((rate, units, secs, gathered))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_partitioned_ensemble():
    """Two gloo ranks each take half of the 256 members: the job counts every member step
    once over the slowest rank's time, and the gathered per-member statistics equal the
    single-process ensemble's in member order."""
    n, world = 256, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29731
    procs = [ctx.Process(target=_worker, args=(r, world, port, n, q)) for r in range(world)]
    for p in procs:
        p.start()
    rate, units, secs, gathered = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert units == 5 * n and abs(secs - 0.2) < 1e-12 and abs(rate - 5 * n / 0.2) < 1e-6
    assert gathered == [_member_size(p) for p in hydrogen_ensemble_params(n)]


def test_gather_rejects_a_wrong_share():
    with pytest.raises(ValueError):
        gather_member_values([1, 2, 3], 10, 1, 0)
    assert gather_member_values(list(range(4)), 4, 1, 0) == [0, 1, 2, 3]
    assert np.isclose(job_throughput(10, 2.0, 1)[0], 5.0)
