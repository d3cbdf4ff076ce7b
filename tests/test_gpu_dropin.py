"""The C++ drop-in entry points on the GPU, called the way the reference's drivers call them.

tests/native/dropin_solve.cpp includes only include/bsj_solver.h, links only libbsj.so,
parses instance files with ``parse_instance`` and calls ``run_gpu_beam_search_v1/_v2``
with a caller-owned ``out_best_sequence`` (gpu/v1/main.cu:50-70).  Every result is
compared with the reference's own gpu kernels (tests/golden/ref_gpu_golden.json): the
makespan bit for bit, and the sequence with the oracle's deterministic schedule when the
result is below 500000; at 500000 or more the sequence buffer must be left untouched
(gpu/v1/solver.cu:280-284).
"""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300 import build as B
from beamsearch_jssp_gpu_gb300.instance import synthetic_instance, write_instance
from oracle import oracle as O

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_gpu_golden.json")


@pytest.fixture(scope="module")
def dropin(tmp_path_factory):
    if not os.path.exists(B.LIB):
        B.build()
    out = str(tmp_path_factory.mktemp("native") / "dropin_solve")
    cxx = shutil.which("g++") or "g++"
    subprocess.check_call([cxx, "-O1", "-std=c++17", "-pthread",
                           os.path.join(ROOT, "tests", "native", "dropin_solve.cpp"), "-o", out,
                           "-L" + B.OUT_DIR, "-lbsj", "-Wl,-rpath," + B.OUT_DIR])
    return out


def _cases(tmp_path):
    with open(GOLDEN) as f:
        recs = [r for r in json.load(f)["records"] if r["K"] <= 1024]
    lines, paths = [], {}
    for r in recs:
        key = (r["n"], r["m"], r["instance_seed"])
        if key not in paths:
            paths[key] = str(tmp_path / ("i_%d_%d_%d.txt" % key))
            write_instance(paths[key], *synthetic_instance(*key))
        lines.append(f'{r["mode"]} {paths[key]} {r["K"]} {r["best_known"]} {r["seed"]}')
    return recs, "\n".join(lines) + "\n"


def _check(recs, outs):
    assert len(outs) == len(recs)
    unwritten = 0
    for r, o in zip(recs, outs):
        assert o["makespan"] == r["makespan"], r
        seq = np.array(o["sequence"], dtype=np.int32)
        if o["makespan"] >= 500000:
            assert (seq == -7).all(), r          # out_best_sequence left untouched
            unwritten += 1
            continue
        mc, du = synthetic_instance(r["n"], r["m"], r["instance_seed"])
        want = O.solve(mc, du, r["mode"], r["K"], r["seed"], best_known=r["best_known"])
        assert np.array_equal(seq, want["seq"]), r
    return unwritten


def test_dropin_entry_points_match_reference_goldens(dropin, tmp_path):
    recs, stdin = _cases(tmp_path)
    p = subprocess.run([dropin], input=stdin, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    outs = [json.loads(x) for x in p.stdout.splitlines()]
    # the golden set holds v1 searches that end with no complete schedule (500000) and
    # searches bounded below their unbounded result
    assert _check(recs, outs) >= 1
    assert any(r["best_known"] < 500000 for r in recs)


def test_dropin_entry_points_from_two_threads(dropin, tmp_path):
    """Two caller threads at once share the per-device context; both see every result."""
    recs, stdin = _cases(tmp_path)
    recs, stdin = recs[:24], "\n".join(stdin.splitlines()[:24]) + "\n"
    p = subprocess.run([dropin, "threads", "2"], input=stdin, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    outs = [json.loads(x) for x in p.stdout.splitlines()]
    _check(recs + recs, outs)
