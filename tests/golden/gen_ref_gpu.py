"""Generate golden vectors from the reference's own gpu kernels (run on a GPU machine).

The reference kernels are compiled from their sources (gpu/v1/solver.cu,
gpu/v2_twophases/solver.cu) into oracle/_ref/ref_gpu_v{1,2}.cubin by ``make -C oracle ref``
where the reference tree exists; oracle/ref_gpu_harness.cpp drives them with the
reference host loop.  Each case runs in a fresh process, twice: the makespan must agree
between the runs; the schedule may not, because several final-level threads copy into
the best-solution buffer at once (gpu/v1/solver.cu:148-154, v2 :126-144).  Instances are
the seeded synthetic generator's, so only (n, m, instance seed) is recorded.

    python tests/golden/gen_ref_gpu.py [OUT.json]                 the base set (80 records)
    python tests/golden/gen_ref_gpu.py --set k4096 --jobs 4 [OUT.json]

``--set k4096`` is the benchmarked configuration: the 50x20 and 100x20 instances of
generator seed 0 at K=4096, search seeds 0-7, unbounded, both solvers (written to
ref_gpu_golden_k4096.json by default).  Its records keep, instead of the reference's
(racy) schedule, its SHA-256 and the makespan the schedule actually has
(``sequence_makespan``, recomputed by the oracle's schedule check); ``--compact RAW.json``
applies that step to a file written with full schedules.  ``--jobs`` runs that many harness processes side by
side (each its own context; they share the one GPU and never wait on one another).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import hashlib
import json
import os
import subprocess
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from beamsearch_jssp_gpu_gb300.instance import synthetic_instance, write_instance  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_build", "ref_gpu_harness")
CUBIN = {v: os.path.join(ROOT, "oracle", "_ref", f"ref_gpu_{v}.cubin") for v in ("v1", "v2")}

# (n, m, instance seed, K, search seeds, best_known list)
CASES = [
    (10, 5, 0, 64, [0, 1, 2, 12345], [500000]),
    (10, 5, 1, 64, [7], [500000]),
    (20, 15, 0, 256, [0, 1, 2, 3], [500000]),
    (20, 15, 1, 1024, [0, 1], [500000]),
    (20, 15, 2, 4096, [0], [500000]),
    (20, 15, 3, 16384, [0], [500000]),
    (6, 4, 5, 8, [3, 4], [500000]),
    (3, 2, 6, 2, [1], [500000]),
    (1, 1, 7, 4, [0], [500000]),
    (5, 1, 8, 4, [0, 9], [500000]),
    (1, 6, 9, 4, [2], [500000]),
    (40, 5, 10, 128, [0, 5], [500000]),
    (50, 20, 11, 256, [0], [500000]),
    (100, 20, 12, 64, [1], [500000]),
]
# the benchmarked configuration: 8 seeds at K=4096 on the 50x20 and 100x20 instances
CASES_K4096 = [
    (50, 20, 0, 4096, list(range(8)), [500000]),
    (100, 20, 0, 4096, list(range(8)), [500000]),
]
# bounded runs: best_known = unbounded result + slack, and = unbounded result (pruned)
BOUND_CASES = [(10, 5, 0, 64, [0, 1]), (20, 15, 0, 256, [0]), (8, 6, 13, 32, [4])]


def compact(records):
    """Schedule -> (SHA-256 of the int32 op ids, makespan of that schedule)."""
    import numpy as np

    from oracle import oracle as O

    out = []
    for r in records:
        r = dict(r)
        seq = np.asarray(r.pop("sequence"), dtype="<i4")
        mc, du = synthetic_instance(r["n"], r["m"], r["instance_seed"])
        r["sequence_sha256"] = hashlib.sha256(seq.tobytes()).hexdigest()
        r["sequence_makespan"] = int(O.schedule_makespan(mc, du, seq)) if r["makespan"] < 500000 else None
        out.append(r)
    return out


def run(mode: str, path: str, K: int, bk: int, seed: int) -> dict:
    out = subprocess.run([HARNESS, mode, CUBIN[mode], path, str(K), str(bk), str(seed)],
                         capture_output=True, text=True, check=True).stdout
    return json.loads(out)


def main(out_path: str, which: str = "base", jobs: int = 1) -> None:
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "gpu-harness"])
    tmp = tempfile.mkdtemp()
    records = []

    def inst_path(n, m, iseed):
        path = os.path.join(tmp, f"i_{n}_{m}_{iseed}.txt")
        if not os.path.exists(path):
            mc, du = synthetic_instance(n, m, iseed)
            write_instance(path, mc, du)
        return path

    def one(n, m, iseed, K, seed, bk, mode):
        path = inst_path(n, m, iseed)
        a = run(mode, path, K, bk, seed)
        b = run(mode, path, K, bk, seed)
        print(mode, n, m, iseed, K, seed, bk, a["makespan"], b["makespan"],
              "same schedule" if a == b else "schedule differs between runs", flush=True)
        return dict(mode=mode, n=n, m=m, instance_seed=iseed, K=K, seed=seed,
                    best_known=bk, makespan=a["makespan"], sequence=a["sequence"],
                    self_consistent=(a == b), makespan_consistent=(a["makespan"] == b["makespan"]))

    def case(n, m, iseed, K, seed, bk):
        base = None
        for mode in ("v1", "v2"):
            r = one(n, m, iseed, K, seed, bk, mode)
            records.append(r)
            if mode == "v1":
                base = r["makespan"]
        return base

    if which == "k4096":
        work = [(n, m, iseed, K, seed, bk, mode) for (n, m, iseed, K, seeds, bks) in CASES_K4096
                for seed in seeds for bk in bks for mode in ("v1", "v2")]
        for (n, m, iseed, *_rest) in work:
            inst_path(n, m, iseed)
        with cf.ThreadPoolExecutor(max_workers=max(1, jobs)) as ex:
            records = compact(list(ex.map(lambda w: one(*w), work)))
    else:
        for (n, m, iseed, K, seeds, bks) in CASES:
            for seed in seeds:
                for bk in bks:
                    case(n, m, iseed, K, seed, bk)
        for (n, m, iseed, K, seeds) in BOUND_CASES:
            for seed in seeds:
                base = case(n, m, iseed, K, seed, 500000)
                for bk in (base + 15, base, base - 10):
                    case(n, m, iseed, K, seed, bk)
    with open(out_path, "w") as f:
        json.dump(dict(generator="tests/golden/gen_ref_gpu.py" + (" --set k4096" if which == "k4096" else ""),
                       source="reference gpu/v1 and gpu/v2_twophases kernels, sm_103a, GB300",
                       records=records), f, indent=0)
    print("wrote", len(records), "records to", out_path)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("out", nargs="?")
    ap.add_argument("--set", dest="which", default="base", choices=["base", "k4096"])
    ap.add_argument("--jobs", type=int, default=1)
    ap.add_argument("--compact", metavar="RAW.json", help="rewrite a k4096 file written with full schedules")
    a = ap.parse_args()
    if a.compact:
        with open(a.compact) as f:
            raw = json.load(f)
        raw["records"] = sorted(compact(raw["records"]), key=lambda r: (r["n"], r["mode"], r["seed"]))
        with open(a.out or os.path.join(ROOT, "tests", "golden", "ref_gpu_golden_k4096.json"), "w") as f:
            json.dump(raw, f, indent=0)
        sys.exit(0)
    name = "ref_gpu_golden.json" if a.which == "base" else "ref_gpu_golden_k4096.json"
    main(a.out or os.path.join(ROOT, "tests", "golden", name), a.which, a.jobs)
