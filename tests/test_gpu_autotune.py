"""The k_step chunk size (survivors per thread block) is a pure work partition: every
size gives the same results, bit for bit, in every mode -- so the autotuner may pick any
of them.  Also: the autotuner's choice is recorded per batch shape and picked up by later
plans of that shape, and a context that tunes on first use solves as before."""
import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300 import BeamSpec, synthetic_instance
from beamsearch_jssp_gpu_gb300 import _native as nat
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _mixed_batch(seed, count, sizes, widths):
    rng = np.random.default_rng(seed)
    insts, beams = [], []
    modes = ["v1", "v2", "clean", "ich", "pms"]
    for k in range(count):
        n, m = sizes[int(rng.integers(0, len(sizes)))]
        insts.append(synthetic_instance(n, m, 300 + k))
        beams.append(BeamSpec(modes[k % 5], int(rng.choice(widths)), 500000, int(rng.integers(0, 2**32)), k, -1))
    return insts, beams


def _same(a, b):
    assert a["makespan"] == b["makespan"]
    assert a["found"] == b["found"]
    assert np.array_equal(a["seq"], b["seq"])
    assert a["expanded"] == b["expanded"]
    assert a["slots"] == b["slots"]
    assert a["levels"] == b["levels"]


def test_every_chunk_size_gives_the_same_results(ctx):
    """Candidates 0 (the default rule), 8, 16, 32 over a mixed-mode batch."""
    # n across the three warp-lane classes (<= 32, <= 64, <= 128); K not multiples of 32
    insts, beams = _mixed_batch(11, 15, [(7, 4), (33, 3), (70, 2), (12, 6)], [1, 5, 24, 100, 257])
    plan = ctx.plan(insts, beams)
    runs = {}
    for ch in nat.CHUNK_CANDIDATES:
        plan.chunk = ch
        assert plan.chunk == ch
        plan.run()
        runs[ch] = plan.results()
    plan.close()
    for ch in nat.CHUNK_CANDIDATES[1:]:
        for a, b in zip(runs[0], runs[ch]):
            _same(a, b)
    for b, r in zip(beams, runs[8]):
        if b.mode in ("ich", "pms") and b.beam_width > 24:
            continue  # keep the oracle's serial heap replay short
        mc, du = insts[b.instance]
        want = O.solve(mc, du, b.mode, b.beam_width, b.seed)
        assert r["makespan"] == want["makespan"], (b, r["makespan"], want["makespan"])
        assert np.array_equal(r["seq"], want["seq"])


@pytest.mark.parametrize("mode", ["v1", "v2", "clean"])
def test_chunk_sizes_agree_on_a_wide_level(ctx, mode):
    mc, du = synthetic_instance(40, 6, 9)
    beams = [BeamSpec(mode, 1000, 500000, 77 + s, 0, 0) for s in range(3)]
    plan = ctx.plan([(mc, du)], beams)
    got = []
    for ch in nat.CHUNK_CANDIDATES:
        plan.chunk = ch
        plan.run()
        got.append(plan.results())
    plan.close()
    for other in got[1:]:
        for a, b in zip(got[0], other):
            _same(a, b)


def test_autotune_picks_a_size_and_records_it_for_the_shape(ctx):
    mc, du = synthetic_instance(20, 15, 4)
    beams = [BeamSpec("v2", 512, 500000, s, 0, 0) for s in range(4)]
    plan = ctx.plan([(mc, du)], beams)
    plan.chunk = 16
    plan.run()
    want = plan.results()
    out = plan.autotune(repeats=1)
    assert out["chunk"] in nat.CHUNK_CANDIDATES
    assert set(out["ms"]) == set(nat.CHUNK_CANDIDATES) and all(v > 0 for v in out["ms"].values())
    assert out["ms"][out["chunk"]] == min(out["ms"].values())
    assert plan.chunk == out["chunk"]
    for a, b in zip(want, plan.results()):
        _same(a, b)
    plan.close()
    # a new plan of the same shape starts with the recorded choice
    again = ctx.plan([synthetic_instance(20, 15, 5)], beams)
    assert again.chunk == out["chunk"]
    again.close()


def test_bad_chunk_size_is_rejected(ctx):
    plan = ctx.plan([synthetic_instance(5, 3, 1)], [BeamSpec("v2", 8, 500000, 1, 0, -1)])
    with pytest.raises(nat.BsjError):
        plan.chunk = 12
    plan.close()


def test_context_that_tunes_on_first_use_solves_the_same():
    from beamsearch_jssp_gpu_gb300 import Context

    insts, beams = _mixed_batch(12, 6, [(9, 5), (36, 4)], [16, 64])
    plain = Context(0)
    want = plain.solve_batch(insts, beams)
    plain.close()
    c = Context(0)
    c.set_autotune(True)
    for _ in range(2):  # first call tunes the shape, the second reuses the tuned plan
        got = c.solve_batch(insts, beams)
        for a, b in zip(want, got):
            _same(a, b)
    c.close()
