"""The multi-GPU path of bench.py is replicas only: each rank solves its own beams and the
job figures are the slowest rank's time and the sum of all ranks' candidates.  Checked
here with two gloo ranks on the CPU (no GPU, no NCCL)."""
import os

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t, u = bench.aggregate_replicas(10.0 + 5 * rank, 1000 * (rank + 1), dist, "cpu")
        seeds = bench.replica_seeds(rank)
        q.put((rank, t, u, seeds))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_aggregate_max_time_and_total_units():
    port = 29000 + os.getpid() % 2000
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    got.sort()
    for rank, t, u, seeds in got:
        assert t == 15.0          # the slower rank's time
        assert u == 3000.0        # both ranks' candidates
        assert seeds == [bench.BEAMS * rank + b for b in range(bench.BEAMS)]
    # the replicas' seeds are disjoint
    assert not set(got[0][3]) & set(got[1][3])


def test_single_process_aggregate_is_local():
    assert bench.aggregate_replicas(12.5, 77, None, "cpu") == (12.5, 77.0)
