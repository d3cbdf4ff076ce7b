"""The benchmarked configuration, bit for bit.

The headline measurement runs 8 beams (search seeds 0-7) of width K=4096 on the 50x20
synthetic instance of generator seed 0, all in one plan; the same is done here for the
50x20 and 100x20 instances, and each beam's result is compared with
  * the reference's own gpu kernels (gpu/v1/solver.cu, gpu/v2_twophases/solver.cu,
    compiled for sm_103a and run on a GB300 by oracle/ref_gpu_harness.cpp;
    tests/golden/ref_gpu_golden_k4096.json from tests/golden/gen_ref_gpu.py --set k4096):
    the makespan;
  * the reference's own CPU solvers (cpu/v1_pms/solver.cpp, cpu/v0_ich/solver.cpp, built
    from their sources; tests/golden/k4096.json "reference_cpu"): the BS-PMS and BS-ICH
    makespan after srand(seed);
  * the oracle (tests/golden/k4096.json "oracle", from tests/golden/gen_k4096.py): the
    makespan, scored children, slots, levels and the SHA-256 of the schedule, in every
    mode.
At this K the selection runs as a cluster of 4 blocks per beam; gpu-v2 is also checked with
the one-block form (the route flags "no_cluster"), so both are pinned at this size.
The 8 beams share one bound group (one device best-makespan word, updated by atomicMin),
as in the measured plan; within a pass every beam prunes against the frozen bound
best_known (500000 here), as the reference does, so the shared word ends as the best of
the 8 makespans without changing any beam's search.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300 import BeamSpec, synthetic_instance

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF_GPU = os.path.join(HERE, "ref_gpu_golden_k4096.json")
CPU_SET = os.path.join(HERE, "k4096.json")
K = 4096
SEEDS = list(range(8))


def _load(path):
    if not os.path.exists(path):
        pytest.skip(f"{os.path.basename(path)} not generated")
    with open(path) as f:
        return json.load(f)


def _sha(seq):
    return hashlib.sha256(np.ascontiguousarray(seq, dtype="<i4").tobytes()).hexdigest()


def _eight_beams(ctx, n, m, mode, flags=(), routes=None):
    """The measured plan: 8 seeded beams of one instance in one set of launches."""
    mc, du = synthetic_instance(n, m, 0)
    plan = ctx.plan([(mc, du)], [BeamSpec(mode, K, 500000, s, 0, 0) for s in SEEDS])
    try:
        if flags:
            plan.set_select_route(*flags)
        plan.run()
        res = plan.results()
        if routes is not None and mode in ("v1", "v2", "clean"):
            routes.update(plan.select_routes())
    finally:
        plan.close()
    if mode in ("v1", "v2", "clean"):
        # the gpu solvers' atomicMin on the shared word (gpu/v1/solver.cu:147-155)
        best = min(r["makespan"] for r in res)
        assert all(r["group_best"] == best for r in res)
    return res


def _oracle_records(mode, n, m):
    recs = {r["seed"]: r for r in _load(CPU_SET)["oracle"] if r["mode"] == mode and (r["n"], r["m"]) == (n, m)}
    assert sorted(recs) == SEEDS
    return recs


def _check_oracle(got, recs, what):
    for s, g in zip(SEEDS, got):
        r = recs[s]
        w = (what, s)
        assert g["makespan"] == r["makespan"], w
        assert g["found"] == r["found"], w
        assert g["expanded"] == r["expanded"], w
        assert g["slots"] == r["slots"], w
        assert g["levels"] == r["levels"], w
        assert _sha(g["seq"]) == r["seq_sha256"], w


@pytest.mark.parametrize("n,m,mode,flags", [(50, 20, "v2", ()), (100, 20, "v2", ()), (50, 20, "v1", ()),
                                            (100, 20, "v1", ()), (50, 20, "v2", ("no_cluster",))])
def test_gpu_modes_match_reference_kernels_and_oracle(ctx, n, m, mode, flags):
    routes = set()
    got = _eight_beams(ctx, n, m, mode, flags, routes)
    assert ("cluster" in routes) == (not flags), sorted(routes)
    ref = {r["seed"]: r for r in _load(REF_GPU)["records"]
           if r["mode"] == mode and (r["n"], r["m"]) == (n, m) and r["K"] == K}
    assert sorted(ref) == SEEDS
    for s, g in zip(SEEDS, got):
        r = ref[s]
        assert r["makespan_consistent"], (n, m, mode, s)
        assert g["makespan"] == r["makespan"], (n, m, mode, s)
        # schedules are compared with the oracle only: the reference's best-solution copy
        # is racy (gpu/v1/solver.cu:148-154), and at this size most of its recorded
        # schedules change between runs or are mixes whose own makespan differs
        # (sequence_makespan in the fixture)
    _check_oracle(got, _oracle_records(mode, n, m), (n, m, mode))


@pytest.mark.parametrize("n,m", [(50, 20), (100, 20)])
def test_clean_mode_matches_oracle(ctx, n, m):
    _check_oracle(_eight_beams(ctx, n, m, "clean"), _oracle_records("clean", n, m), (n, m, "clean"))


@pytest.mark.parametrize("n,m,mode", [(50, 20, "pms"), (100, 20, "pms"), (50, 20, "ich")])
def test_cpu_modes_match_reference_cpu_solvers(ctx, n, m, mode):
    """BS-PMS / BS-ICH mode (srand(seed) rand() streams, libstdc++ bounded heap) against the
    reference's own CPU solver after srand(seed), and against the oracle."""
    got = _eight_beams(ctx, n, m, mode)
    ref = {r["seed"]: r["makespan"] for r in _load(CPU_SET)["reference_cpu"]
           if r["mode"] == mode and (r["n"], r["m"]) == (n, m)}
    assert sorted(ref) == SEEDS
    for s, g in zip(SEEDS, got):
        assert g["makespan"] == ref[s], (n, m, mode, s)
    _check_oracle(got, _oracle_records(mode, n, m), (n, m, mode))
