"""The allocation-free entry point (bsj_solve_noalloc) against the ordinary one.

bsj_solve_noalloc exists for callers that must not allocate device memory -- operator or
plugin hosts whose device memory belongs to the host framework, and latency-critical
loops where a cudaMalloc could synchronise the device or fail mid-run.  It keeps all of
its intermediate state in one library-owned scratch array, so consecutive calls reuse
(and must fully re-initialise) the same memory: the test calls it twice in a row per case
and compares each result with bsj_solve's, bit for bit.  The test's own input/output
buffers are allocated here, by the caller, as such a host framework would.

This file sorts last so that a run stopping at its first failure has run every other
test first; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300 import Context, synthetic_instance
from beamsearch_jssp_gpu_gb300 import _native as nat

pytestmark = pytest.mark.gpu

BSJ_ERR_LIMIT = 2


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_matches_solve_on_two_consecutive_calls():
    torch = pytest.importorskip("torch")
    lib = nat.load()
    ctx = Context(0)
    # K=100 and K=1 leave the last 16-survivor chunk partial
    cases = [((20, 10, 7), "v2", 256, 3), ((10, 5, 0), "v2", 64, 0), ((33, 4, 2), "clean", 512, 9),
             ((50, 20, 1), "v2", 1024, 5), ((20, 10, 7), "v2", 100, 4), ((15, 8, 3), "clean", 100, 1),
             ((12, 6, 4), "v2", 1, 2)]
    for (n, m, iseed), mode, K, seed in cases:
        mc, du = synthetic_instance(n, m, iseed)
        want = ctx.solve(mc, du, mode, K, seed)
        d_mc = torch.tensor(mc, dtype=torch.int32, device="cuda")
        d_du = torch.tensor(du, dtype=torch.int32, device="cuda")
        for call in range(2):
            out = torch.full((2 + n * m,), -7, dtype=torch.int32, device="cuda")
            st = lib.bsj_solve_noalloc(n, m, _vp(d_mc), _vp(d_du), nat.MODES[mode], K, 500000, seed,
                                       _vp(out), None)
            assert st == nat.BSJ_OK, (n, m, mode, K, call, st)
            torch.cuda.synchronize()
            o = out.cpu().numpy()
            assert o[0] == want["makespan"], (n, m, mode, K, call)
            assert o[1] == int(want["found"])
            assert np.array_equal(o[2:], want["seq"]), (n, m, mode, K, call)
    ctx.close()


def test_noalloc_invalid_instances_then_a_valid_call():
    """An invalid instance gives makespan -1, found 0 and a zero sequence in the caller's
    buffer; the scratch keeps that state, so the next valid call must still equal
    bsj_solve."""
    torch = pytest.importorskip("torch")
    lib = nat.load()
    ctx = Context(0)
    n, m = 16, 10
    mc, du = synthetic_instance(n, m, 11)
    bad_machine = mc.copy()
    bad_machine[3, 4] = m                       # machine id outside [0, m)
    bad_duration = du.copy()
    bad_duration[7, 2] = 1 << 24                # duration outside [0, 2^24)
    overflow = np.full_like(du, (1 << 24) - 1)  # 160 such durations sum past 2^31-1
    want = ctx.solve(mc, du, "v2", 100, 6)
    for bad_mc, bad_du in ((bad_machine, du), (mc, bad_duration), (mc, overflow)):
        d_mc = torch.tensor(bad_mc, dtype=torch.int32, device="cuda")
        d_du = torch.tensor(bad_du, dtype=torch.int32, device="cuda")
        out = torch.full((2 + n * m,), -7, dtype=torch.int32, device="cuda")
        st = lib.bsj_solve_noalloc(n, m, _vp(d_mc), _vp(d_du), nat.MODES["v2"], 100, 500000, 6, _vp(out), None)
        assert st == nat.BSJ_OK
        torch.cuda.synchronize()
        o = out.cpu().numpy()
        assert o[0] == -1 and o[1] == 0 and not o[2:].any()
        d_mc = torch.tensor(mc, dtype=torch.int32, device="cuda")
        d_du = torch.tensor(du, dtype=torch.int32, device="cuda")
        st = lib.bsj_solve_noalloc(n, m, _vp(d_mc), _vp(d_du), nat.MODES["v2"], 100, 500000, 6, _vp(out), None)
        assert st == nat.BSJ_OK
        torch.cuda.synchronize()
        o = out.cpu().numpy()
        assert o[0] == want["makespan"] and o[1] == int(want["found"])
        assert np.array_equal(o[2:], want["seq"])
    ctx.close()


def test_noalloc_on_a_caller_stream():
    torch = pytest.importorskip("torch")
    lib = nat.load()
    ctx = Context(0)
    mc, du = synthetic_instance(20, 15, 2)
    want = ctx.solve(mc, du, "clean", 300, 8)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        d_mc = torch.tensor(mc, dtype=torch.int32, device="cuda")
        d_du = torch.tensor(du, dtype=torch.int32, device="cuda")
        out = torch.zeros(2 + mc.size, dtype=torch.int32, device="cuda")
        st = lib.bsj_solve_noalloc(20, 15, _vp(d_mc), _vp(d_du), nat.MODES["clean"], 300, 500000, 8, _vp(out),
                                   ctypes.c_void_p(stream.cuda_stream))
        assert st == nat.BSJ_OK
    stream.synchronize()
    o = out.cpu().numpy()
    assert o[0] == want["makespan"] and np.array_equal(o[2:], want["seq"])
    ctx.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = nat.load()
    n, m = 100, 20
    d_mc = torch.zeros(n * m, dtype=torch.int32, device="cuda")
    out = torch.zeros(2 + n * m, dtype=torch.int32, device="cuda")
    # the per-level history alone (n*m*K*4 bytes) exceeds the 64 MiB scratch
    st = lib.bsj_solve_noalloc(n, m, _vp(d_mc), _vp(d_mc), nat.MODES["v2"], 16384, 500000, 0, _vp(out), None)
    assert st == BSJ_ERR_LIMIT
    st = lib.bsj_solve_noalloc(4, 3, _vp(d_mc), _vp(d_mc), nat.MODES["v2"], 16385, 500000, 0, _vp(out), None)
    assert st == BSJ_ERR_LIMIT
