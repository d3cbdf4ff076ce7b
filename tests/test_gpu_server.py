"""The serving loop (bsj_server_*): each result is the same alone and in the mix.

Requests of mixed shapes and modes arrive from two threads while others run; the server
admits them as slots and memory free up, runs them concurrently, and reuses plans by
shape.  Every result must equal the plain one-at-a-time solve (bsj_solve) bit for bit:
makespan, found, schedule, expanded children and levels.
"""
import random
import threading
import time

import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300 import BsjError, Server, synthetic_instance
from beamsearch_jssp_gpu_gb300 import _native as nat

pytestmark = pytest.mark.gpu


def _requests(count, seed):
    rng = random.Random(seed)
    out = []
    for i in range(count):
        n = rng.choice([10, 15, 20, 30])
        m = rng.choice([5, 10, 15])
        mode = rng.choice(["v1", "v2", "clean", "v2", "clean", "pms", "ich"])
        K = rng.choice([16, 32, 64]) if mode in ("pms", "ich") else rng.choice([64, 256, 1024])
        mc, du = synthetic_instance(n, m, 1000 + i)
        out.append(dict(mc=mc, du=du, mode=mode, K=K, seed=rng.randrange(1 << 31)))
    return out


def _same(a, b):
    assert a["makespan"] == b["makespan"]
    assert a["found"] == b["found"]
    assert a["expanded"] == b["expanded"] and a["levels"] == b["levels"]
    if a["found"]:
        assert np.array_equal(a["seq"], b["seq"])


def _submit_from_threads(srv, reqs, nthreads=2):
    tickets = [None] * len(reqs)

    def worker(k):
        rng = random.Random(k)
        for i in range(k, len(reqs), nthreads):
            r = reqs[i]
            tickets[i] = srv.submit(r["mc"], r["du"], r["mode"], r["K"], r["seed"])
            time.sleep(rng.random() * 0.002)

    th = [threading.Thread(target=worker, args=(k,)) for k in range(nthreads)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    return tickets


def test_results_same_alone_and_in_the_mix(ctx):
    reqs = _requests(40, 7)
    alone = [ctx.solve(r["mc"], r["du"], r["mode"], r["K"], r["seed"]) for r in reqs]
    with Server(0, max_inflight=6) as srv:
        tickets = _submit_from_threads(srv, reqs)
        got = [srv.wait(t) for t in tickets]
        st = srv.stats()
    for a, g in zip(alone, got):
        _same(a, g)
        assert g["queue_ms"] >= 0 and g["run_ms"] > 0
    assert st["submitted"] == st["completed"] == len(reqs)
    assert 1 <= st["peak_inflight"] <= 6
    assert st["plans_reused"] > 0
    assert st["plans_built"] + st["plans_reused"] == len(reqs)


@pytest.mark.parametrize("cluster_inflight", [1, -1, 100])
def test_wide_requests_in_either_select_form(ctx, cluster_inflight):
    """K=4096 requests: the server gives each the cluster select only while at most
    cluster_inflight others run (1: some with, some without; -1: never; 100: always).
    Every result equals the plain solve."""
    reqs = []
    for i in range(8):
        mc, du = synthetic_instance(20, 15, 2000 + i)
        reqs.append(dict(mc=mc, du=du, mode=("v2", "clean", "v1")[i % 3], K=4096, seed=17 + i))
    alone = [ctx.solve(r["mc"], r["du"], r["mode"], r["K"], r["seed"]) for r in reqs]
    with Server(0, max_inflight=4, cluster_inflight=cluster_inflight) as srv:
        tickets = _submit_from_threads(srv, reqs)
        got = [srv.wait(t) for t in tickets]
    for a, g in zip(alone, got):
        _same(a, g)


def test_memory_budget_bounds_what_the_device_holds(ctx):
    reqs = _requests(24, 11)
    sizes = [ctx.estimate([(r["mc"], r["du"])], [_beam(r)]) for r in reqs]
    budget = int(max(sizes) * 2.5)
    alone = [ctx.solve(r["mc"], r["du"], r["mode"], r["K"], r["seed"]) for r in reqs]
    with Server(0, max_inflight=8, memory_budget=budget) as srv:
        tickets = _submit_from_threads(srv, reqs, nthreads=3)
        got = [srv.wait(t) for t in tickets]
        st = srv.stats()
    for a, g in zip(alone, got):
        _same(a, g)
    assert st["budget_bytes"] == budget
    assert st["peak_device_bytes"] <= budget


def _beam(r):
    from beamsearch_jssp_gpu_gb300 import BeamSpec

    return BeamSpec(r["mode"], r["K"], nat.NO_BOUND, r["seed"])


def test_poll_is_nonblocking_and_tickets_retire(ctx):
    mc, du = synthetic_instance(50, 20, 3)
    with Server(0, max_inflight=2) as srv:
        t = srv.submit(mc, du, "v2", 4096, 5)
        first = srv.poll(t)
        deadline = time.time() + 60
        res = first
        while res is None and time.time() < deadline:
            time.sleep(0.001)
            res = srv.poll(t)
        assert res is not None
        _same(ctx.solve(mc, du, "v2", 4096, 5), res)
        with pytest.raises(BsjError):
            srv.poll(t)  # retired
        with pytest.raises(BsjError):
            srv.poll(123456789)


def test_rejections_at_submit():
    mc, du = synthetic_instance(10, 5, 1)
    bad = mc.copy()
    bad[0, 0] = 7  # machine id outside [0, m)
    with Server(0, max_inflight=2, memory_budget=1 << 20) as srv:
        with pytest.raises(BsjError) as e:
            srv.submit(bad, du, "v2", 64, 0)
        assert e.value.status == nat.BSJ_ERR_INVALID
        with pytest.raises(BsjError) as e:
            srv.submit(mc, du, "v2", 16384, 0)  # needs more than the 1 MiB budget
        assert e.value.status == nat.BSJ_ERR_LIMIT
        with pytest.raises(BsjError) as e:
            srv.submit(mc, du, "v2", 0, 0)
        assert e.value.status == nat.BSJ_ERR_LIMIT
        t = srv.submit(mc, du, "v2", 64, 0)
        assert srv.wait(t)["found"]


def test_prepared_plans_are_reused_by_later_requests(ctx):
    """bsj_server_prepare builds plans of a shape before traffic; requests of that shape then
    report built_plan = 0, a request of another shape builds its plan (built_plan = 1), and
    every result still equals the plain solve."""
    mc, du = synthetic_instance(20, 10, 5)
    other = synthetic_instance(15, 5, 6)
    with Server(0, max_inflight=4) as srv:
        srv.prepare(mc, du, "v2", 256, copies=3)
        deadline = time.time() + 60
        while srv.stats()["plans_prepared"] < 3:
            assert time.time() < deadline, "prepared plans not built within a minute"
            time.sleep(0.01)
        assert srv.stats()["plans_built"] == 3 and srv.stats()["completed"] == 0
        tickets = [srv.submit(synthetic_instance(20, 10, 50 + k)[0], synthetic_instance(20, 10, 50 + k)[1], "v2",
                              256, k) for k in range(3)]
        got = [srv.wait(t) for t in tickets]
        assert not any(g["built_plan"] for g in got)
        for k, g in enumerate(got):
            _same(g, ctx.solve(*synthetic_instance(20, 10, 50 + k), "v2", 256, k))
        g = srv.wait(srv.submit(*other, "clean", 64, 9))
        assert g["built_plan"]
        _same(g, ctx.solve(*other, "clean", 64, 9))
        st = srv.stats()
        assert st["plans_built"] == 4 and st["plans_reused"] == 3 and st["completed"] == 4
