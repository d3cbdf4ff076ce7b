"""CUDA path == oracle, bit for bit (makespan, schedule, counters), through the C ABI."""
import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300 import BeamSpec, BsjError, synthetic_instance
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MODES = ["v1", "v2", "clean", "ich", "pms"]
SMALL = [  # (n, m, K, instance seed)
    (10, 5, 64, 0), (10, 5, 64, 1), (6, 4, 8, 2), (3, 2, 2, 3), (1, 1, 4, 4), (5, 1, 4, 5),
    (1, 6, 3, 6), (12, 3, 1, 7), (20, 15, 256, 8), (40, 5, 128, 9), (33, 4, 64, 10),
    (64, 3, 32, 11), (100, 4, 16, 12), (128, 2, 8, 13), (8, 64, 16, 14),
]


def check(ctx, mc, du, mode, K, seed, bk=500000):
    got = ctx.solve(mc, du, mode, K, seed, bk)
    want = O.solve(mc, du, mode, K, seed, best_known=bk)
    assert got["makespan"] == want["makespan"], (mode, K, seed, bk, got["makespan"], want["makespan"])
    assert got["found"] == want["found"]
    assert np.array_equal(got["seq"], want["seq"]), (mode, K, seed, bk)
    assert got["expanded"] == want["expanded"], (mode, got["expanded"], want["expanded"])
    if mode in ("v1", "v2", "clean"):
        assert got["slots"] == want["slots"]
    assert got["levels"] == want["levels"]
    return got


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("n,m,K,iseed", SMALL)
def test_small_instances_match_oracle(ctx, mode, n, m, K, iseed):
    mc, du = synthetic_instance(n, m, iseed)
    for seed in (0, 12345 + iseed):
        check(ctx, mc, du, mode, K, seed)


@pytest.mark.parametrize("mode", MODES)
def test_bounds_match_oracle(ctx, mode):
    mc, du = synthetic_instance(10, 5, 21)
    base = O.solve(mc, du, mode, 64, 3)["makespan"]
    for bk in (base + 30, base + 1, base, base - 20, 1):
        check(ctx, mc, du, mode, 64, 3, bk)


@pytest.mark.parametrize("mode", MODES)
def test_seeds_near_wraparound(ctx, mode):
    mc, du = synthetic_instance(8, 5, 22)
    for seed in (2**31 - 3, 2**32 - 2, 2**31 + 7):
        check(ctx, mc, du, mode, 32, seed)


@pytest.mark.parametrize("mode", ["v1", "v2", "clean", "pms"])
def test_medium_instance(ctx, mode):
    mc, du = synthetic_instance(20, 15, 1)
    check(ctx, mc, du, mode, 512, 5)


def test_wide_beam_ich(ctx):
    mc, du = synthetic_instance(15, 5, 2)
    check(ctx, mc, du, "ich", 1000, 12345)


def test_schedules_verify(ctx):
    mc, du = synthetic_instance(30, 10, 3)
    for mode in MODES:
        r = ctx.solve(mc, du, mode, 128, 1)
        assert r["found"]
        assert O.schedule_makespan(mc, du, r["seq"]) == r["makespan"]


def test_invalid_inputs_raise_without_running(ctx):
    mc, du = synthetic_instance(4, 3, 0)
    with pytest.raises(BsjError):
        ctx.solve(mc, du, "v2", 0, 0)
    with pytest.raises(BsjError):
        ctx.solve(mc, du, "v2", 16385, 0)
    bad = mc.copy()
    bad[0, 0] = 3
    with pytest.raises(BsjError):
        ctx.solve(bad, du, "v2", 8, 0)
    neg = du.copy()
    neg[1, 1] = -1
    with pytest.raises(BsjError):
        ctx.solve(mc, neg, "v2", 8, 0)
    big = synthetic_instance(129, 2, 0)
    with pytest.raises(BsjError):
        ctx.solve(*big, "v2", 8, 0)
    with pytest.raises(BsjError):
        ctx.solve_batch([(mc, du)], [BeamSpec("v2", 8, 500000, 0, 3)])
    # the context stays usable
    check(ctx, mc, du, "v2", 8, 0)


@pytest.mark.parametrize("mode", ["v1", "v2", "clean"])
@pytest.mark.parametrize("n,m,K", [(64, 3, 2048), (40, 5, 4096), (30, 6, 8192)])
def test_large_levels_match_oracle(ctx, mode, n, m, K):
    """Levels with more candidate keys than the select stages in shared memory (25-35 K per
    level here), which run the chunk-walking select with 32-bit dense-rank keys."""
    mc, du = synthetic_instance(n, m, 3)
    check(ctx, mc, du, mode, K, 5)


@pytest.mark.parametrize("mode", ["ich", "pms"])
@pytest.mark.parametrize("K", [8192, 9000])
def test_wide_heaps_match_oracle(ctx, mode, K):
    """ICH/PMS beams whose bounded heap fills to K=8192 and K=9000 (4-5 M children offered
    over 60 levels): the replay of libstdc++'s heap steps stays exact at these widths."""
    mc, du = synthetic_instance(12, 5, 3)
    check(ctx, mc, du, mode, K, 77)
