"""Multi-beam launches: seeds as beams, uneven instances, mixed modes, shared bounds,
multi-start iterations -- each result equal to the single-beam solve / the oracle."""
import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300 import BeamSpec, synthetic_instance
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_seeds_as_beams_equal_single_solves(ctx):
    mc, du = synthetic_instance(20, 10, 1)
    beams = [BeamSpec("v2", 256, 500000, s, 0, 0) for s in range(8)]
    batch = ctx.solve_batch([(mc, du)], beams)
    for s, r in enumerate(batch):
        single = ctx.solve(mc, du, "v2", 256, s)
        assert r["makespan"] == single["makespan"]
        assert np.array_equal(r["seq"], single["seq"])
        assert r["expanded"] == single["expanded"]
    # the shared bound word ends at the best of the group
    assert all(r["group_best"] == min(x["makespan"] for x in batch) for r in batch)


def test_uneven_mixed_batch_equals_oracle(ctx):
    rng = np.random.default_rng(5)
    insts, beams = [], []
    modes = ["v1", "v2", "clean", "ich", "pms"]
    for k in range(24):
        n = int(rng.choice([3, 5, 8, 10, 33]))
        m = int(rng.choice([1, 2, 4, 5]))
        insts.append(synthetic_instance(n, m, 100 + k))
        beams.append(BeamSpec(modes[k % 5], int(rng.choice([1, 4, 16, 64])), 500000, int(rng.integers(0, 2**32)), k, -1))
    res = ctx.solve_batch(insts, beams)
    for b, r in zip(beams, res):
        mc, du = insts[b.instance]
        want = O.solve(mc, du, b.mode, b.beam_width, b.seed)
        assert r["makespan"] == want["makespan"], (b, r["makespan"], want["makespan"])
        assert np.array_equal(r["seq"], want["seq"])
        assert r["expanded"] == want["expanded"]


def test_beams_sharing_instances(ctx):
    a = synthetic_instance(10, 5, 1)
    b = synthetic_instance(15, 4, 2)
    beams = [BeamSpec("v1", 32, 500000, 1, 0), BeamSpec("v2", 64, 500000, 2, 1),
             BeamSpec("pms", 16, 500000, 3, 0), BeamSpec("ich", 16, 500000, 4, 1)]
    res = ctx.solve_batch([a, b], beams)
    for bm, r in zip(beams, res):
        mc, du = (a, b)[bm.instance]
        assert r["makespan"] == O.solve(mc, du, bm.mode, bm.beam_width, bm.seed)["makespan"]


@pytest.mark.parametrize("mode", ["v1", "v2", "clean"])
def test_iterations_carry_the_bound(ctx, mode):
    """gpu/v1/main.cu:58-71 with 3 ranks: every round uses the best of earlier rounds."""
    mc, du = synthetic_instance(10, 5, 3)
    seeds = np.arange(12, dtype=np.uint32).reshape(4, 3) * 7919 + 11
    best, seq, rounds = ctx.solve_iterations(mc, du, mode, 32, seeds)
    want = O.solve_iterations(mc, du, mode, 32, seeds, 4)
    assert best == want["best"]
    assert np.array_equal(rounds, want["round_best"])
    assert O.schedule_makespan(mc, du, seq) == best
    assert np.array_equal(seq, want["seq"])


@pytest.mark.parametrize("mode", ["pms", "ich"])
@pytest.mark.parametrize("n,m,K,beams,iters", [(10, 5, 32, 3, 4), (20, 10, 64, 2, 3), (15, 15, 128, 4, 2)])
def test_iterations_continue_the_rand_stream(ctx, mode, n, m, K, beams, iters):
    """cpu/v1_pms/main.cpp:56-67: each rank seeds rand() once and its later rounds draw
    on from where the previous pass stopped."""
    mc, du = synthetic_instance(n, m, 5)
    seeds = np.arange(beams, dtype=np.uint32) * 104729 + 3
    best, seq, rounds = ctx.solve_iterations(mc, du, mode, K, seeds, iterations=iters)
    want = O.solve_iterations(mc, du, mode, K, seeds, iters)
    assert best == want["best"]
    assert np.array_equal(rounds, want["round_best"])
    if best < 500000:
        assert O.schedule_makespan(mc, du, seq) == best


def test_plan_rerun_is_deterministic(ctx):
    mc, du = synthetic_instance(20, 10, 4)
    beams = [BeamSpec("v2", 512, 500000, s, 0, 0) for s in range(4)]
    plan = ctx.plan([(mc, du)], beams)
    plan.run()
    first = plan.results()
    plan.run()
    plan.run()
    again = plan.results()
    for x, y in zip(first, again):
        assert x["makespan"] == y["makespan"] and np.array_equal(x["seq"], y["seq"])
    assert plan.launches > 0
    plan.close()


@pytest.mark.parametrize("groups", ["1", "3"])
def test_beam_group_count_does_not_change_results(ctx, monkeypatch, groups):
    """BSJ_MAX_BEAM_GROUPS (how many beam groups run as concurrent graph branches) and the
    longest-first segment layout change scheduling only: every beam's result stays the
    same, in the caller's order."""
    rng = np.random.default_rng(9)
    insts, beams = [], []
    for k in range(10):
        insts.append(synthetic_instance(int(rng.choice([5, 12, 20])), int(rng.choice([3, 6, 10])), 300 + k))
        beams.append(BeamSpec(["v2", "clean", "v1", "pms"][k % 4], 64, 500000, 1000 + k, k, -1))
    want = ctx.solve_batch(insts, beams)
    monkeypatch.setenv("BSJ_MAX_BEAM_GROUPS", groups)
    plan = ctx.plan(insts, beams)
    plan.run()
    got = plan.results()
    plan.close()
    for w, g, b in zip(want, got, beams):
        assert g["makespan"] == w["makespan"], b
        assert np.array_equal(g["seq"], w["seq"])
        assert g["expanded"] == w["expanded"] and g["levels"] == w["levels"]
