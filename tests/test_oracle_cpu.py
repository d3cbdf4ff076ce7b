"""The CPU oracle pinned against the reference (no GPU needed).

* glibc rand() restatement == libc rand()
* ICH / PMS restatements == the reference's own CPU solvers compiled from their sources
  (oracle/_ref/libref_cpu.so; present where the reference tree is, skipped elsewhere)
* gpu-mode restatements == the reference's gpu kernels (tests/golden/ref_gpu_golden.json,
  produced on a GB300 by tests/golden/gen_ref_gpu.py)
"""
import ctypes
import json
import os

import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300.instance import synthetic_instance, write_instance
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_gpu_golden.json")
needs_ref = pytest.mark.skipif(not O.ref_cpu_available(), reason="reference CPU build absent")


@pytest.mark.parametrize("seed", [0, 1, 12345, 2**31 - 1, 2**31 + 5, 2**32 - 1])
def test_glibc_rand_matches_libc(seed):
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(ctypes.c_uint(seed))
    want = [libc.rand() for _ in range(3000)]
    assert O.glibc_rand(seed, 3000).tolist() == want


SIZES = [(10, 5, 64), (6, 4, 8), (15, 5, 100), (8, 8, 32), (5, 1, 4), (3, 2, 2), (1, 1, 3), (1, 5, 2), (12, 3, 1)]


@needs_ref
@pytest.mark.parametrize("n,m,K", SIZES)
def test_oracle_ich_matches_reference(tmp_path, n, m, K):
    for iseed in range(3):
        mc, du = synthetic_instance(n, m, iseed)
        path = str(tmp_path / f"i{iseed}.txt")
        write_instance(path, mc, du)
        for seed in (12345, iseed, 99 + iseed):
            assert O.solve(mc, du, "ich", K, seed)["makespan"] == O.ref_ich(path, K, seed)


@needs_ref
@pytest.mark.parametrize("n,m,K", SIZES)
def test_oracle_pms_matches_reference(tmp_path, n, m, K):
    for iseed in range(3):
        mc, du = synthetic_instance(n, m, iseed)
        path = str(tmp_path / f"i{iseed}.txt")
        write_instance(path, mc, du)
        for seed in (0, 7 + iseed):
            base = O.ref_pms(path, K, 500000, seed)
            assert O.solve(mc, du, "pms", K, seed)["makespan"] == base
            for bk in (base + 25, base, base - 5):
                assert O.solve(mc, du, "pms", K, seed, best_known=bk)["makespan"] == O.ref_pms(path, K, bk, seed)


@needs_ref
def test_oracle_pms_larger_matches_reference(tmp_path):
    mc, du = synthetic_instance(20, 15, 4)
    path = str(tmp_path / "i.txt")
    write_instance(path, mc, du)
    for seed in (0, 1):
        assert O.solve(mc, du, "pms", 256, seed)["makespan"] == O.ref_pms(path, 256, 500000, seed)


@needs_ref
def test_oracle_pms_iterations_match_reference(tmp_path):
    # srand once, then rounds that continue the rand() stream with the carried bound
    # (cpu/v1_pms/main.cpp:56-67 with one rank)
    for (n, m, iseed, K) in ((8, 4, 3, 16), (12, 6, 5, 32), (15, 10, 1, 64)):
        mc, du = synthetic_instance(n, m, iseed)
        path = str(tmp_path / f"i{iseed}.txt")
        write_instance(path, mc, du)
        for seed in (0, 11):
            for iters in (1, 2, 5):
                got = O.solve_iterations(mc, du, "pms", K, [seed], iters)
                assert got["best"] == O.ref_pms_iterations(path, K, seed, iters), (n, m, seed, iters)
                assert O.schedule_makespan(mc, du, got["seq"]) == got["best"]


def test_oracle_iterations_compose_single_solves():
    # gpu modes: round r's beams are independent solves bounded by the earlier rounds' best
    mc, du = synthetic_instance(10, 5, 2)
    seeds = np.array([[3, 9], [4, 10], [5, 11]], dtype=np.uint32)
    for mode in ("v1", "v2", "clean"):
        got = O.solve_iterations(mc, du, mode, 32, seeds, 3)
        bound = 500000
        for it in range(3):
            spans = [O.solve(mc, du, mode, 32, int(seeds[it, b]), best_known=bound)["makespan"] for b in range(2)]
            bound = min([bound] + spans)
            assert got["round_best"][it] == bound, (mode, it)
        assert got["best"] == bound
    # ICH/PMS: the first round equals plain solves with the srand seeds
    for mode in ("ich", "pms"):
        got = O.solve_iterations(mc, du, mode, 32, [7, 8], 1)
        assert got["best"] == min(O.solve(mc, du, mode, 32, s)["makespan"] for s in (7, 8))


@pytest.mark.parametrize("mode", ["ich", "pms", "v1", "v2", "clean"])
def test_oracle_schedules_verify(mode):
    for iseed in range(3):
        mc, du = synthetic_instance(9, 4, iseed)
        r = O.solve(mc, du, mode, 16, iseed)
        assert r["found"]
        assert O.schedule_makespan(mc, du, r["seq"]) == r["makespan"]


def test_oracle_m1_reference_quirk():
    """With m == 1 the reference reads op_finish[op-1] of the previous job
    (jssp_types.h:82): jobs then run back to back even on different machines."""
    mc = np.zeros((4, 1), dtype=np.int32)
    du = np.array([[3], [5], [2], [4]], dtype=np.int32)
    r = O.solve(mc, du, "v2", 8, 0)
    assert r["makespan"] == 14


def _golden():
    if not os.path.exists(GOLDEN):
        pytest.skip("reference gpu goldens not generated yet")
    with open(GOLDEN) as f:
        return json.load(f)["records"]


def test_golden_makespans_deterministic():
    recs = _golden()
    assert len(recs) >= 60
    for r in recs:
        assert r.get("makespan_consistent", True)


def classify_reference_sequence(mc, du, r, oracle_run):
    """'equal' (the deterministic choice: min cmax, lowest slot), 'tie' (another complete
    child with the same makespan), 'corrupt' (the racy copy mixed several children: the
    schedule does not reach the reported makespan) -- anything else is a parity failure."""
    ref = np.array(r["sequence"], dtype=np.int32)
    if np.array_equal(ref, oracle_run["seq"]):
        return "equal"
    if any(np.array_equal(ref, t) for t in oracle_run.get("tie_seqs", [])):
        return "tie"
    if O.schedule_makespan(mc, du, ref) != r["makespan"]:
        return "corrupt"
    return "unexplained"


@pytest.mark.parametrize("mode", ["v1", "v2"])
def test_oracle_gpu_modes_match_reference_kernels(mode):
    """The gpu-mode restatement reproduces the reference gpu kernels' makespan exactly;
    every reference schedule is explained (equal / tie / corrupted by the racy copy)."""
    recs = [r for r in _golden() if r["mode"] == mode and r["K"] <= 4096]
    assert recs
    kinds = {}
    for r in recs:
        mc, du = synthetic_instance(r["n"], r["m"], r["instance_seed"])
        got = O.solve(mc, du, mode, r["K"], r["seed"], best_known=r["best_known"], max_ties=4096)
        assert got["makespan"] == r["makespan"], r
        if r["makespan"] >= 500000:
            continue
        k = classify_reference_sequence(mc, du, r, got)
        assert k != "unexplained", r
        kinds[k] = kinds.get(k, 0) + 1
    assert kinds.get("equal", 0) > 0


# ---- the benchmarked configuration: 50x20 / 100x20, K=4096, search seeds 0-7 ----------
K4096 = os.path.join(os.path.dirname(__file__), "golden", "k4096.json")
REF_GPU_K4096 = os.path.join(os.path.dirname(__file__), "golden", "ref_gpu_golden_k4096.json")


def _k4096():
    with open(K4096) as f:
        cpu = json.load(f)
    with open(REF_GPU_K4096) as f:
        gpu = json.load(f)
    return {(r["mode"], r["n"], r["seed"]): r for r in cpu["oracle"]}, cpu["reference_cpu"], gpu["records"]


def test_k4096_oracle_records_equal_the_references():
    """The committed oracle records at the benchmarked size equal every makespan of the
    reference's own CPU solvers (BS-PMS 50x20 and 100x20, BS-ICH 50x20, 24 searches) and of
    its gpu kernels run on a GB300 (v1 and v2, 50x20 and 100x20, 32 searches)."""
    orc, ref_cpu, ref_gpu = _k4096()
    assert len(ref_cpu) == 24 and len(ref_gpu) == 32
    for r in ref_cpu:
        assert orc[(r["mode"], r["n"], r["seed"])]["makespan"] == r["makespan"], r
    for r in ref_gpu:
        assert r["makespan_consistent"], r
        assert orc[(r["mode"], r["n"], r["seed"])]["makespan"] == r["makespan"], r


def _oracle_job(args):
    mode, n, m, seed = args
    mc, du = synthetic_instance(n, m, 0)
    r = O.solve(mc, du, mode, 4096, seed)
    import hashlib

    return (int(r["makespan"]), int(r["expanded"]), int(r["slots"]), int(r["levels"]),
            hashlib.sha256(np.ascontiguousarray(r["seq"], dtype="<i4").tobytes()).hexdigest())


def test_k4096_oracle_reruns_match_its_records_and_the_reference():
    """Three searches of the 50x20 benchmarked instance rerun here (BS-PMS seeds 0 and 1,
    gpu-v2 seed 0), in parallel processes: each equals its committed record and the
    reference's own result for it."""
    import multiprocessing as mp

    orc, ref_cpu, ref_gpu = _k4096()
    jobs = [("pms", 50, 20, 0), ("pms", 50, 20, 1), ("v2", 50, 20, 0)]
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        out = pool.map(_oracle_job, jobs)
    ref = {(r["mode"], r["n"], r["seed"]): r["makespan"] for r in ref_cpu + ref_gpu}
    for (mode, n, m, seed), (mk, ex, sl, lv, sha) in zip(jobs, out):
        rec = orc[(mode, n, seed)]
        assert (mk, ex, sl, lv, sha) == (rec["makespan"], rec["expanded"], rec["slots"], rec["levels"],
                                         rec["seq_sha256"])
        assert mk == ref[(mode, n, seed)]
