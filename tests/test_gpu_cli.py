"""The command-line drivers (beamsearch_jssp_gpu_gb300/cli/bsj_cli.cpp) end to end on the
GPU, against the oracle's multi-start loop with the same rand() seeds.

Each driver's MPI ranks are beams of one launch; with ``--seed S`` rank r seeds rand()
with S + r, so the expected makespans follow from the oracle:
  exec_gpu_v1/v2  round seeds = rank r's successive rand() draws (gpu/v1/main.cu:58-71)
  BS-PMS          rank r's rand() stream continued across rounds (cpu/v1_pms/main.cpp:56-67)
  BS-ICH          srand(12345), one pass (cpu/v0_ich/main.cpp:39-41)
"""
import csv
import os
import re
import subprocess

import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300 import build as B
from beamsearch_jssp_gpu_gb300.instance import synthetic_instance, write_instance
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    if not os.path.exists(B.CLI_BIN):
        B.build()


def _cli(name, *args, cwd=None):
    r = subprocess.run([os.path.join(B.OUT_DIR, name), *map(str, args)], capture_output=True, text=True,
                       cwd=cwd, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout


def _best(out):
    return int(re.search(r"Best Makespan\s*:\s*(\d+)", out).group(1))


def _rank_draws(base, ranks, iters):
    return np.stack([O.glibc_rand(base + r, iters) for r in range(ranks)], axis=1).astype(np.uint32)


@pytest.mark.parametrize("name,mode", [("exec_gpu_v1", "v1"), ("exec_gpu_v2", "v2")])
def test_exec_gpu_matches_oracle_loop(tmp_path, name, mode):
    mc, du = synthetic_instance(12, 6, 4)
    path = tmp_path / "inst.txt"
    write_instance(str(path), mc, du)
    sched = tmp_path / "best.csv"
    out = _cli(name, path, 48, 3, "--ranks", 2, "--seed", 5, "--schedule", sched)
    assert "Beam Width (K): 48  |  MPI Ranks: 2" in out and "Iterations: 3" in out
    assert "Execution Time :" in out
    want = O.solve_iterations(mc, du, mode, 48, _rank_draws(5, 2, 3), 3)
    assert _best(out) == want["best"]
    rows = list(csv.DictReader(open(sched)))
    assert len(rows) == 12 * 6
    assert max(int(r["finish"]) for r in rows) == want["best"]
    seq = [(int(r["job"]) - 1) * 6 + int(r["step"]) for r in rows]
    assert O.schedule_makespan(mc, du, np.array(seq, dtype=np.int32)) == want["best"]


def test_bs_pms_matches_oracle_loop(tmp_path):
    mc, du = synthetic_instance(10, 5, 6)
    path = tmp_path / "inst.txt"
    write_instance(str(path), mc, du)
    out = _cli("BS-PMS", path, 24, "--ranks", 3, "--seed", 9, "--iters", 12)
    want = O.solve_iterations(mc, du, "pms", 24, [9, 10, 11], 12)
    assert _best(out) == want["best"]
    lines = re.findall(r"iter\s+(\d+) \| global best = (\d+)", out)
    assert [int(i) for i, _ in lines] == [0, 10]
    assert [int(v) for _, v in lines] == [want["round_best"][0], want["round_best"][10]]


def test_bs_ich_matches_oracle(tmp_path):
    mc, du = synthetic_instance(8, 4, 1)
    path = tmp_path / "inst.txt"
    write_instance(str(path), mc, du)
    out = _cli("BS-ICH", path, 16)
    assert "Scheduled Ops    : 32" in out
    assert _best(out) == O.solve(mc, du, "ich", 16, 12345)["makespan"]


@pytest.mark.parametrize("name,mode,iters", [("exec_gpu_v1_bench", "v1", 2), ("BS-PMS-bench", "pms", 2)])
def test_suites_resolve_ids_and_print_rows(tmp_path, name, mode, iters):
    insts = {"01": synthetic_instance(5, 3, 1), "11": synthetic_instance(6, 4, 2)}
    for i, (mc, du) in insts.items():
        write_instance(str(tmp_path / f"la{i}.txt"), mc, du)
    out = _cli(name, "--ids", "01,11,99", "--iters", iters, "--seed", 4, cwd=str(tmp_path))
    assert "SKIP la99  (file not found)" in out
    rows = {}
    for line in out.splitlines():
        f = line.split()
        if len(f) == 7 and f[0].isdigit():
            rows[f[1]] = f
    for i, (mc, du) in insts.items():
        f = rows[f"./la{i}.txt"]
        K = 1000 if i == "01" else 5000
        assert int(f[0]) == K and int(f[2]) == mc.shape[0] and int(f[4]) == mc.size + 2
        seeds = [4] if mode == "pms" else _rank_draws(4, 1, iters)
        assert int(f[5]) == O.solve_iterations(mc, du, mode, K, seeds, iters)["best"], i


def test_time_width_sweep(tmp_path):
    mc, du = synthetic_instance(6, 3, 7)
    write_instance(str(tmp_path / "la10.txt"), mc, du)
    out = _cli("exec_cpu_time_width", "--ids", "10", "--iters", 1, "--seed", 2, cwd=str(tmp_path))
    widths = [int(line.split()[0]) for line in out.splitlines() if line.split() and line.split()[0].isdigit()]
    assert widths == [100, 200, 400, 800, 1600, 3200, 6400, 12800, 25600]
    assert "width above the engine's limit" in out
    for w, line in enumerate(l for l in out.splitlines() if l.split() and l.split()[0].isdigit()):
        f = line.split()
        if int(f[0]) > 16384:
            continue
        assert int(f[5]) == O.solve_iterations(mc, du, "pms", int(f[0]), [2 + w], 1)["best"]
