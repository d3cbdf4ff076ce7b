"""Every route of the top-K selection, forced, against the oracle.

The selection kernel replaces the reference's full stable sort of all child slots
(cub::DeviceRadixSort::SortPairs, gpu/v1/solver.cu:255-258, gpu/v2_twophases/solver.cu:
336-339).  By level size it normally takes the direct staged pass or bucket compaction +
dense-rank sort; the radix-select, raw-LSD, rank-LSD, bitonic and large-level routes run
only on rare or large levels.  Beams of K >= 4096 run it as a cluster of 2 blocks (4 where
K * n >= 150 000): the bucket + dense-rank route split over the blocks on levels of more
than 4 096 keys, the one-block routes as its fallback.
bsj_plan_set_select_route forces them onto small levels,
and each forced search must equal the oracle bit for bit (makespan, schedule, scored
children, slots, levels) -- where a wrong tie order would show -- and must report that
the forced route ran (bsj_plan_select_routes).

Instances with durations in {1, 2} or {1, 2, 3} make many children share a makespan, so
many keys share a score up to the hashed noise term and the stable (score, slot) order
decides.
"""
import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300 import BeamSpec, synthetic_instance
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# (forced flags, routes that must have run)
SMALL_ROUTES = [
    ((), {"direct"}),
    (("force_large",), {"large"}),
    (("no_direct",), {"bucket", "dense"}),
    (("no_direct", "no_dense"), {"bucket", "raw_lsd"}),
    (("no_direct", "rank_lsd"), {"bucket", "rank_lsd"}),
    (("no_direct", "bitonic"), {"bucket", "bitonic"}),
    (("radix",), {"radix", "raw_lsd"}),
    (("radix", "bitonic"), {"radix", "bitonic"}),
    (("force_cluster",), {"cluster"}),
]
# levels wider than the shared-memory staging area (more than 16 384 candidate keys)
LARGE_ROUTES = [
    ((), {"large"}),
    (("no_large",), {"bucket", "dense"}),
    (("no_large", "no_dense"), {"bucket", "raw_lsd"}),
    (("no_large", "rank_lsd"), {"bucket", "rank_lsd"}),
    (("no_large", "bitonic"), {"bucket", "bitonic"}),
    (("no_large", "radix"), {"radix", "raw_lsd"}),
    (("no_large", "radix", "bitonic"), {"radix", "bitonic"}),
    # up to 32 768 keys: staged over the two blocks of the cluster
    (("force_cluster",), {"cluster"}),
]


def tie_instance(n, m, seed, dmax):
    """Job-wise machine permutations, durations uniform in [1, dmax]."""
    rng = np.random.default_rng(seed)
    mc = np.stack([rng.permutation(m) for _ in range(n)]).astype(np.int32)
    du = rng.integers(1, dmax + 1, size=(n, m)).astype(np.int32)
    return mc, du


SMALL_CASES = [
    ("ties 12x4 K=64", tie_instance(12, 4, 1, 2), 64, 3),
    ("ties 20x6 K=200", tie_instance(20, 6, 2, 2), 200, 5),
    ("ties 30x5 K=1000", tie_instance(30, 5, 3, 3), 1000, 7),
    ("synthetic 8x8 K=37", synthetic_instance(8, 8, 4), 37, 11),
    ("ties 40x1 K=50", tie_instance(40, 1, 5, 2), 50, 2),
]


def _run(ctx, mc, du, mode, K, seed, flags):
    plan = ctx.plan([(mc, du)], [BeamSpec(mode, K, 500000, seed, 0, -1)])
    try:
        plan.set_select_route(*flags)
        plan.run()
        res = plan.results()[0]
        routes = plan.select_routes()
    finally:
        plan.close()
    return res, routes


def _same(got, want, what):
    assert got["makespan"] == want["makespan"], what
    assert got["expanded"] == want["expanded"], what
    assert got["slots"] == want["slots"], what
    assert got["levels"] == want["levels"], what
    assert np.array_equal(got["seq"], want["seq"]), what


@pytest.mark.parametrize("mode", ["v1", "v2", "clean"])
def test_forced_routes_small_levels(ctx, mode):
    for name, (mc, du), K, seed in SMALL_CASES:
        want = O.solve(mc, du, mode, K, seed)
        for flags, must in SMALL_ROUTES:
            got, routes = _run(ctx, mc, du, mode, K, seed, flags)
            what = (name, mode, flags, sorted(routes))
            _same(got, want, what)
            assert must <= routes, what


@pytest.mark.parametrize("mode", ["v2", "clean", "v1"])
def test_forced_routes_large_levels(ctx, mode):
    """120x4 at K=768: about 30 candidates per parent, so levels carry more than 16 384
    keys and the selection reads them in place (the large-level route, or with it
    excluded the unstaged general path)."""
    mc, du = synthetic_instance(120, 4, 6)
    K, seed = 768, 9
    want = O.solve(mc, du, mode, K, seed)
    for flags, must in LARGE_ROUTES:
        got, routes = _run(ctx, mc, du, mode, K, seed, flags)
        what = (mode, flags, sorted(routes))
        _same(got, want, what)
        assert must <= routes, what


@pytest.mark.parametrize("mode", ["v2", "clean"])
def test_forced_routes_wide_beam(ctx, mode):
    """K=16384 (more survivors than the 8 192-key radix buffer): normally the large-level
    route; with it excluded, the MSD radix select and the 16 384-key bitonic sort; in the
    cluster form (launched by default at this K), the one-block routes on its first block."""
    mc, du = synthetic_instance(16, 3, 3)
    want = O.solve(mc, du, mode, 16384, 0)
    for flags, must in (((), {"large"}), (("no_large",), {"radix", "bitonic"}),
                        (("no_cluster",), {"large"})):
        got, routes = _run(ctx, mc, du, mode, 16384, 0, flags)
        what = (mode, flags, sorted(routes))
        _same(got, want, what)
        assert must <= routes, what


@pytest.mark.parametrize("mode", ["v2", "v1"])
def test_cluster_route_default_and_off(ctx, mode):
    """K=4096 on 20x15 (levels of up to ~15 000 keys): the cluster route by default (levels
    of at most 8 192 keys take the one-block routes on its first block), the one-block
    bucket route with the cluster form off; both equal the oracle."""
    mc, du = synthetic_instance(20, 15, 1)
    want = O.solve(mc, du, mode, 4096, 5)
    for flags, must, never in (((), {"cluster"}, set()), (("no_cluster",), {"bucket"}, {"cluster"})):
        got, routes = _run(ctx, mc, du, mode, 4096, 5, flags)
        what = (mode, flags, sorted(routes))
        _same(got, want, what)
        assert must <= routes and not (never & routes), what


@pytest.mark.parametrize("mode", ["v2", "v1"])
def test_forced_cluster_four_blocks(ctx, mode):
    """K * n >= 150 000 launches 4 blocks per beam; forced onto every level (down to levels
    of a few keys, where most blocks hold none), on tie-heavy durations, it equals the
    oracle."""
    for mc, du, seed in ((tie_instance(40, 5, 9, 2)[0], tie_instance(40, 5, 9, 2)[1], 3),
                         (*synthetic_instance(40, 4, 5), 8)):
        want = O.solve(mc, du, mode, 4096, seed)
        for flags in (("force_cluster",), ()):
            got, routes = _run(ctx, mc, du, mode, 4096, seed, flags)
            what = (mode, flags, sorted(routes))
            _same(got, want, what)
            if flags:
                assert "cluster" in routes, what


def test_select_cluster_switch(ctx):
    """bsj_plan_set_select_cluster: one thread block per beam and back, each form's graph
    kept; the result never changes."""
    mc, du = synthetic_instance(20, 15, 1)
    want = O.solve(mc, du, "v2", 4096, 5)
    plan = ctx.plan([(mc, du)], [BeamSpec("v2", 4096, 500000, 5, 0, -1)])
    try:
        for on in (True, False, True, False):
            plan.set_select_cluster(on)
            plan.run()
            got = plan.results()[0]
            routes = plan.select_routes()
            _same(got, want, (on, sorted(routes)))
            assert ("cluster" in routes) == on, (on, sorted(routes))
    finally:
        plan.close()


def test_route_flags_rejected(ctx):
    mc, du = synthetic_instance(6, 3, 0)
    plan = ctx.plan([(mc, du)], [BeamSpec("v2", 8, 500000, 0, 0, -1)])
    try:
        with pytest.raises(Exception):
            plan.set_select_route("force_large", "no_large")
        with pytest.raises(Exception):
            plan.set_select_route("force_cluster", "no_cluster")
        from beamsearch_jssp_gpu_gb300 import _native as nat

        assert plan.lib.bsj_plan_set_select_route(plan.h, 1 << 9) == nat.BSJ_ERR_INVALID
        assert plan.lib.bsj_plan_set_select_route(plan.h, 1 << 10) == nat.BSJ_ERR_INVALID
    finally:
        plan.close()
