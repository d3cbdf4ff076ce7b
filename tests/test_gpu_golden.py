"""CUDA path == the reference's own gpu kernels (goldens from tests/golden/gen_ref_gpu.py,
run on a GB300 with the reference kernels compiled from their sources)."""
import json
import os

import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300 import synthetic_instance
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_gpu_golden.json")


def _records():
    if not os.path.exists(GOLDEN):
        pytest.skip("reference gpu goldens not generated yet")
    with open(GOLDEN) as f:
        return json.load(f)["records"]


@pytest.mark.parametrize("mode", ["v1", "v2"])
def test_makespan_and_schedule_match_reference_kernels(ctx, mode):
    """Makespan bit-exact against the reference kernels; the schedule equals the oracle's
    deterministic choice, and the reference's own schedule is that one, another tie, or
    a mix produced by its racy best-solution copy (gpu/v1/solver.cu:148-154)."""
    recs = [r for r in _records() if r["mode"] == mode]
    assert recs
    for r in recs:
        mc, du = synthetic_instance(r["n"], r["m"], r["instance_seed"])
        got = ctx.solve(mc, du, mode, r["K"], r["seed"], r["best_known"])
        assert got["makespan"] == r["makespan"], r
        if r["K"] > 4096:
            continue  # oracle too slow at this width; makespan parity only
        want = O.solve(mc, du, mode, r["K"], r["seed"], best_known=r["best_known"], max_ties=4096)
        assert np.array_equal(got["seq"], want["seq"])
        if r["makespan"] < 500000:
            ref = np.array(r["sequence"], dtype=np.int32)
            explained = (np.array_equal(ref, got["seq"])
                         or any(np.array_equal(ref, t) for t in want["tie_seqs"])
                         or O.schedule_makespan(mc, du, ref) != r["makespan"])
            assert explained, r
