"""Full-size workloads (50x20 / 100x20, K=4096, 8 seeds as beams): size-independent
properties -- every returned schedule is a feasible permutation whose recomputed makespan
equals the reported one, reruns are identical, a beam in the batch equals the same beam
alone, and the 8-beam bound word is the minimum."""
import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300 import BeamSpec, synthetic_instance
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,m", [(50, 20), (100, 20)])
def test_eight_seed_beams_full_size(ctx, n, m):
    mc, du = synthetic_instance(n, m, 0)
    beams = [BeamSpec("v2", 4096, 500000, s, 0, 0) for s in range(8)]
    plan = ctx.plan([(mc, du)], beams)
    plan.run()
    res = plan.results()
    plan.run()
    again = plan.results()
    plan.close()
    for r, r2 in zip(res, again):
        assert r["found"]
        assert O.schedule_makespan(mc, du, r["seq"]) == r["makespan"]
        assert r2["makespan"] == r["makespan"] and np.array_equal(r2["seq"], r["seq"])
        assert r["levels"] == n * m
    best = min(r["makespan"] for r in res)
    assert all(r["group_best"] == best for r in res)
    alone = ctx.solve(mc, du, "v2", 4096, 5)
    assert alone["makespan"] == res[5]["makespan"] and np.array_equal(alone["seq"], res[5]["seq"])


@pytest.mark.parametrize("mode", ["v1", "clean", "pms"])
def test_full_size_other_modes_feasible(ctx, mode):
    mc, du = synthetic_instance(50, 20, 1)
    r = ctx.solve(mc, du, mode, 1024, 3)
    assert r["found"]
    assert O.schedule_makespan(mc, du, r["seq"]) == r["makespan"]


@pytest.mark.parametrize("mode", ["clean", "v2"])
def test_k16384_select_path(ctx, mode):
    """K=16384 with ~100k keys per level (more than the register path holds) against the
    oracle."""
    mc, du = synthetic_instance(16, 3, 3)
    got = ctx.solve(mc, du, mode, 16384, 0)
    want = O.solve(mc, du, mode, 16384, 0)
    assert got["makespan"] == want["makespan"]
    assert np.array_equal(got["seq"], want["seq"])
    assert got["expanded"] == want["expanded"]
