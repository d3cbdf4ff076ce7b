"""The lane-group k_step forms against the oracle, bit for bit.

k_step_g materialises and expands each survivor with a group of 4 lanes (forms 1, 2) or
8 lanes (forms 3, 4), the parent snapshot staged in shared memory by the group's 16-byte
copies (1, 3) or by one bulk copy completing on an mbarrier (2, 4).  Each is run over the parity suite's shapes -- every ready-list lane
class up to n = 128, m = 1 (the jobs-chain quirk), K = 1, K not a multiple of 32 --
with bounds that prune children and early levels where fewer children are scored than
min(P*n, K), so that v2's filler ranks take both of their paths: a pruned child that is
materialised anyway, and a branch that does not exist, whose rank keeps the ping-pong
buffer's old content (gpu/v2_twophases/solver.cu:191).
"""
import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300 import BeamSpec, synthetic_instance
from beamsearch_jssp_gpu_gb300 import _native as nat
from oracle import oracle as O

FORMS = nat.GROUP_FORMS

pytestmark = pytest.mark.gpu

SHAPES = [  # (n, m, K, instance seed)
    (10, 5, 64, 0), (6, 4, 8, 2), (3, 2, 2, 3), (1, 1, 4, 4), (5, 1, 4, 5), (1, 6, 3, 6), (12, 3, 1, 7),
    (20, 15, 256, 8), (40, 5, 128, 9), (33, 4, 64, 10), (64, 3, 32, 11), (100, 4, 16, 12), (128, 2, 8, 13),
    (8, 64, 16, 14), (50, 20, 100, 15), (30, 10, 1000, 16),
]


def _solve(ctx, mc, du, mode, K, seed, bk, form):
    plan = ctx.plan([(mc, du)], [BeamSpec(mode, K, bk, seed, 0, -1)])
    try:
        plan.chunk = form
        plan.run()
        return plan.results()[0]
    finally:
        plan.close()


def _check(ctx, mc, du, mode, K, seed, bk=500000):
    want = O.solve(mc, du, mode, K, seed, best_known=bk)
    for form in FORMS:
        got = _solve(ctx, mc, du, mode, K, seed, bk, form)
        what = (form, mode, mc.shape, K, seed, bk)
        assert got["makespan"] == want["makespan"], what
        assert got["found"] == want["found"], what
        assert np.array_equal(got["seq"], want["seq"]), what
        assert got["expanded"] == want["expanded"], what
        assert got["slots"] == want["slots"], what
        assert got["levels"] == want["levels"], what


@pytest.mark.parametrize("mode", ["v2", "clean"])
@pytest.mark.parametrize("n,m,K,iseed", SHAPES)
def test_group_forms_match_oracle(ctx, mode, n, m, K, iseed):
    mc, du = synthetic_instance(n, m, iseed)
    for seed in (0, 2**32 - 2 - iseed):
        _check(ctx, mc, du, mode, K, seed)


@pytest.mark.parametrize("mode", ["v2", "clean"])
def test_group_forms_with_bounds(ctx, mode):
    mc, du = synthetic_instance(10, 5, 21)
    base = O.solve(mc, du, mode, 64, 3)["makespan"]
    for bk in (base + 30, base + 1, base, base - 20, 1):
        _check(ctx, mc, du, mode, 64, 3, bk)


def test_group_form_in_a_batch_with_other_modes(ctx):
    """A plan mixing modes and instances: beam groups holding only v2/clean beams run the
    lane-group form, the others the warp form of the same chunk size; every beam equals its
    own oracle solve."""
    insts = [synthetic_instance(12, 4, 1), synthetic_instance(30, 6, 2), synthetic_instance(70, 3, 3)]
    beams = [BeamSpec(mode, K, 500000, 100 + i, i % 3, -1)
             for i, (mode, K) in enumerate([("v2", 64), ("clean", 100), ("v1", 50), ("ich", 16), ("v2", 33),
                                            ("pms", 8), ("clean", 257), ("v2", 512)])]
    plan = ctx.plan(insts, beams)
    try:
        for form in FORMS:
            plan.chunk = form
            plan.run()
            for b, r in zip(beams, plan.results()):
                mc, du = insts[b.instance]
                want = O.solve(mc, du, b.mode, b.beam_width, b.seed)
                assert r["makespan"] == want["makespan"], (form, b)
                assert np.array_equal(r["seq"], want["seq"]), (form, b)
                assert r["expanded"] == want["expanded"], (form, b)
    finally:
        plan.close()


@pytest.mark.parametrize("mode", ["v2", "clean"])
def test_group_forms_wide_beam(ctx, mode):
    """K=16384 on 16x3 (~100 K candidate keys per level: the large-level select) with each
    group form against the oracle."""
    mc, du = synthetic_instance(16, 3, 3)
    want = O.solve(mc, du, mode, 16384, 0)
    for form in FORMS:
        got = _solve(ctx, mc, du, mode, 16384, 0, 500000, form)
        what = (form, mode)
        assert got["makespan"] == want["makespan"], what
        assert np.array_equal(got["seq"], want["seq"]), what
        assert got["expanded"] == want["expanded"] and got["slots"] == want["slots"], what
