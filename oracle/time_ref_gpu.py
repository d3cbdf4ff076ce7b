"""Device time of the reference's own gpu solvers on this GPU (TEST INFRASTRUCTURE).

Runs oracle/ref_gpu_harness (the reference's kernels from gpu/v1/solver.cu and
gpu/v2_twophases/solver.cu, compiled from their sources into oracle/_ref/*.cubin by
``make -C oracle ref``) with its ``time`` option on seeded synthetic instances and prints
one JSON line per case: the summed CUDA-event time of the reference's two kernels per
search, the host time of the harness's substituted sort, and the makespan.  The kernel
time is a lower bound of the reference's GPU time: its cub::DeviceRadixSort over all P*n
slots per level (gpu/v1/solver.cu:255-258) comes on top.  Each case runs in a fresh
process, as the reference's results assume.

    python oracle/time_ref_gpu.py            # needs a GPU, the cubins and make
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from beamsearch_jssp_gpu_gb300.instance import synthetic_instance, write_instance  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(HERE, "_build", "ref_gpu_harness")
CUBIN = {v: os.path.join(HERE, "_ref", f"ref_gpu_{v}.cubin") for v in ("v1", "v2")}

# (n, m, instance seed, K, search seed)
CASES = [(20, 15, 0, 1024, 0), (50, 20, 0, 4096, 0)]


def main() -> int:
    subprocess.check_call(["make", "-s", "-C", HERE, "gpu-harness"])
    with tempfile.TemporaryDirectory() as tmp:
        for n, m, iseed, K, seed in CASES:
            mc, du = synthetic_instance(n, m, iseed)
            path = os.path.join(tmp, f"syn_{n}x{m}_{iseed}.txt")
            write_instance(path, mc, du)
            for mode in ("v2", "v1"):
                t0 = time.perf_counter()
                out = subprocess.run([HARNESS, mode, CUBIN[mode], path, str(K), "500000", str(seed), "time"],
                                     capture_output=True, text=True, check=True).stdout
                wall = time.perf_counter() - t0
                d = json.loads(out)
                print(json.dumps({"solver": f"reference gpu {mode}", "jobs": n, "machines": m, "beam_width": K,
                                  "seed": seed, "levels": n * m, "kernel_ms": d["kernel_ms"],
                                  "kernel_ms_total": sum(d["kernel_ms"]), "host_sort_ms": d["host_sort_ms"],
                                  "wall_s": wall, "makespan": d["makespan"]}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
