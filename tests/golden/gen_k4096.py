"""Golden records for the benchmarked configuration (generated on the CPU).

The benchmarked configuration is the 50x20 and 100x20 synthetic instances of generator
seed 0 at beam width K=4096 with search seeds 0-7 (the eight MPI ranks of BS-PMS become
eight beams of one launch).  This script writes ``k4096.json`` next to itself with

* ``oracle``: the CPU oracle (oracle/bsj_oracle.c, pinned to the reference) for every
  mode -- makespan, found, expanded (scored children), slots, levels and the SHA-256 of
  the best schedule (int32 little-endian op ids) -- so the GPU tests compare the full
  search at this size without running the oracle for minutes;
* ``reference_cpu``: the reference's own CPU solvers (cpu/v1_pms/solver.cpp,
  cpu/v0_ich/solver.cpp, compiled from their sources into oracle/_ref/libref_cpu.so by
  ``make -C oracle ref``), makespan per seed after ``srand(seed)``.  These pin the
  oracle's ICH/PMS records at this size (tests/test_oracle_cpu.py checks the two agree).

    python tests/golden/gen_k4096.py [--procs 8]

About 15 minutes on 8 cores.  The oracle in v1 mode keeps every child slot in the
reference's state layout (about 6.8 GB at 100x20), so those runs get a smaller pool.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import multiprocessing as mp
import os
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

K = 4096
SEEDS = list(range(8))
SHAPES = [(50, 20, 0), (100, 20, 0)]
# oracle modes per shape; ICH at 100x20 is left out (its serial heap makes the GPU test
# take minutes there)
ORACLE_MODES = {(50, 20): ["v1", "v2", "clean", "pms", "ich"], (100, 20): ["v1", "v2", "clean", "pms"]}
REF_SOLVERS = {(50, 20): ["pms", "ich"], (100, 20): ["pms"]}


def seq_sha256(seq) -> str:
    import numpy as np

    return hashlib.sha256(np.ascontiguousarray(seq, dtype="<i4").tobytes()).hexdigest()


def _oracle_job(args):
    n, m, iseed, mode, seed = args
    from beamsearch_jssp_gpu_gb300.instance import synthetic_instance
    from oracle import oracle as O

    mc, du = synthetic_instance(n, m, iseed)
    t0 = time.perf_counter()
    r = O.solve(mc, du, mode, K, seed)
    rec = dict(mode=mode, n=n, m=m, instance_seed=iseed, K=K, seed=seed, best_known=500000,
               makespan=int(r["makespan"]), found=bool(r["found"]), expanded=int(r["expanded"]),
               slots=int(r["slots"]), levels=int(r["levels"]), seq_sha256=seq_sha256(r["seq"]))
    print("oracle", mode, n, m, seed, rec["makespan"], f"{time.perf_counter() - t0:.1f}s", flush=True)
    return rec


def _ref_job(args):
    n, m, iseed, solver, seed, path = args
    from oracle import oracle as O

    t0 = time.perf_counter()
    mk = O.ref_pms(path, K, 500000, seed) if solver == "pms" else O.ref_ich(path, K, seed)
    print("reference", solver, n, m, seed, mk, f"{time.perf_counter() - t0:.1f}s", flush=True)
    return dict(solver="cpu/v1_pms" if solver == "pms" else "cpu/v0_ich", mode=solver, n=n, m=m,
                instance_seed=iseed, K=K, seed=seed, best_known=500000, makespan=int(mk))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--procs", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--out", default=os.path.join(HERE, "k4096.json"))
    a = ap.parse_args()
    from beamsearch_jssp_gpu_gb300.instance import synthetic_instance, write_instance
    from oracle import oracle as O

    O.build(ref=False)
    if not O.ref_cpu_available():
        sys.exit("oracle/_ref/libref_cpu.so is missing: build it with `make -C oracle ref`")
    tmp = tempfile.mkdtemp()
    paths = {}
    for (n, m, iseed) in SHAPES:
        paths[(n, m)] = os.path.join(tmp, f"i_{n}_{m}_{iseed}.txt")
        write_instance(paths[(n, m)], *synthetic_instance(n, m, iseed))

    big = [(n, m, i, "v1", s) for (n, m, i) in SHAPES if n * m >= 2000 for s in SEEDS]
    small = [(n, m, i, md, s) for (n, m, i) in SHAPES for md in ORACLE_MODES[(n, m)] for s in SEEDS
             if (n, m, i, md, s) not in big]
    refs = [(n, m, i, sv, s, paths[(n, m)]) for (n, m, i) in SHAPES for sv in REF_SOLVERS[(n, m)]
            for s in SEEDS]
    ctx = mp.get_context("spawn")
    with ctx.Pool(a.procs) as pool:
        ref_async = pool.map_async(_ref_job, refs)
        oracle_small = pool.map(_oracle_job, small)
        reference = ref_async.get()
    with ctx.Pool(max(1, min(a.procs, 4))) as pool:
        oracle_big = pool.map(_oracle_job, big)
    with open(a.out, "w") as f:
        json.dump(dict(generator="tests/golden/gen_k4096.py", K=K, seeds=SEEDS,
                       instances=[dict(n=n, m=m, instance_seed=i) for (n, m, i) in SHAPES],
                       oracle=oracle_small + oracle_big, reference_cpu=reference), f, indent=0)
    print("wrote", a.out)


if __name__ == "__main__":
    main()
