#!/usr/bin/env python
"""Benchmark: expanded candidates/s of the beam-search level path at K=4096, 50x20.

Workload (one "step"): a full search -- all n*m = 1000 levels -- of 8 independently
seeded beams (seeds 8*rank .. 8*rank+7) of width K=4096 on one synthetic 50x20 instance
(machine permutation per job, durations U[1,99], int32; generator seed 0), gpu-v2 mode
(pivot-machine branching, fp32 score, two-phase score-then-materialise), all 8 beams in
one set of launches sharing a device best-makespan word.  Metric = scored children
(valid, unpruned) summed over levels and beams / step time.

Arms:
  (default)          libbsj.so on the GPU: ``value`` device-timed with the instance
                     resident, ``e2e`` through the C ABI from host buffers.
  --impl reference   the reference's own CPU implementation of machine-focused beam search,
                     BS-PMS (cpu/v1_pms/solver.cpp: glibc rand() pivots, fp64 score,
                     libstdc++ bounded heap), as the oracle port pinned bit for bit to it,
                     one process per beam on the host cores, each step a full 1 000-level
                     search of the 8 beams.  The reference has no CPU implementation of its
                     gpu-v2 semantics; the same workload in those semantics on the host
                     cores is the default arm's ``cpu_baseline`` (the matched comparison).

Also on the JSON line (rank 0; --no-extras skips them):
  "cpu_baseline"      the oracle's restatement of gpu/v2_twophases (the headline's own
             algorithm) over the same 8 beams, all 1 000 levels, a process per beam;
  "cpu_baseline_pms"  the BS-PMS port (what --impl reference times) on the same beams;
  "matched_ratios"    GPU over CPU in the same semantics: value and e2e over cpu_baseline,
             pms_exact over cpu_baseline_pms;
  "pms_exact" the same 8 beams in BS-PMS mode (the reference CPU solver's exact semantics,
             serial bounded heap per beam), candidates/s and makespans;
  "batched"  256 synthetic instances of uneven size (n in {10..100}, m in {5..20},
             K in {256..4096}) in one bsj_solve_batch, solves/s against the same
             instances solved one call at a time (the plain path), makespans compared; the
             batch's k_step chunk sizes are autotuned on its first call (untimed);
  "serving"  400 requests with Poisson arrivals through bsj_server (continuous
             batching) at 150/s (sustained) and 1000/s (overload), solves/s and p50/p99
             latency per rate (also split by requests that reused / built a plan) against
             the plain path on the same requests, results compared; plans of every shape
             are prepared before the timed streams;
  "serving_mixed_branching"  96 requests, half BS-ICH / BS-PMS (K=256), half gpu-v2 /
             clean, at 40/s: solves/s, p50/p99 overall and per mode, results compared.

Multi-GPU: replicas only (each rank runs its own 8 beams; no collective on the data
path); value = all ranks' candidates / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_JOBS, N_MACH, K, BEAMS, MODE, INSTANCE_SEED = 50, 20, 4096, 8, "v2", 0
METRIC = "expanded candidates/s at K=4096 50x20"
UNIT = "candidates/s"
CPU_SAMPLE_LEVELS = 1000       # levels per beam in one CPU sample (a full 50x20 search)
L2_FLUSH_BYTES = 512 << 20     # > 129 MB L2


def _config(world: int, mode: str = MODE) -> dict:
    what = {"v2": "pivot-machine beam search, gpu/v2_twophases semantics (hashed pivot and noise, fp32 score, "
                  "stable top-K sort)",
            "pms": "BS-PMS, cpu/v1_pms semantics (glibc rand() pivot and noise, fp64 score, libstdc++ bounded "
                   "heap)"}[mode]
    return {"workload": f"{what}, {N_JOBS}x{N_MACH} synthetic (seed {INSTANCE_SEED}), K={K}, {BEAMS} seeded "
                        f"beams per GPU, all {N_JOBS * N_MACH} levels",
            "jobs": N_JOBS, "machines": N_MACH, "beam_width": K, "beams_per_gpu": BEAMS, "mode": mode,
            "levels": N_JOBS * N_MACH, "parallelism": f"replicas x{world}",
            "l2": "flushed between timed steps (512 MB write); per-level working set ~26 MB stays L2-resident "
                  "within a step"}


# ------------------------------------------------------------------------------------
# CPU side: the oracle (pinned bit for bit to the reference) on the host cores
# ------------------------------------------------------------------------------------
CPU_KIND = {"v2": "oracle restatement of gpu/v2_twophases/solver.cu (the headline's semantics)",
            "pms": "oracle port of cpu/v1_pms/solver.cpp (pinned to the reference)"}


def _cpu_worker(args):
    n, m, iseed, width, mode, seed, levels = args
    from beamsearch_jssp_gpu_gb300.instance import synthetic_instance
    from oracle import oracle as O

    mc, du = synthetic_instance(n, m, iseed)
    t0 = time.perf_counter()
    r = O.solve(mc, du, mode, width, seed, max_levels=levels)
    return r["expanded"], time.perf_counter() - t0


def cpu_sample(procs: int, seeds, levels: int = CPU_SAMPLE_LEVELS, pool=None, mode: str = "pms") -> dict:
    """One bounded sample on the host cores, a process per beam (`pool`: reuse an open
    spawn pool of `procs` workers)."""
    from oracle import oracle as O

    if pool is None:
        O.build(ref=False)
        with mp.get_context("spawn").Pool(procs) as own:
            return cpu_sample(procs, seeds, levels, own, mode)
    t0 = time.perf_counter()
    out = pool.map(_cpu_worker, [(N_JOBS, N_MACH, INSTANCE_SEED, K, mode, s, levels) for s in seeds])
    wall = time.perf_counter() - t0
    expanded = sum(e for e, _ in out)
    busy = max(t for _, t in out)
    return dict(expanded=expanded, wall=wall, busy=busy, value=expanded / busy)


def cpu_baseline_entry(r: dict, procs: int, mode: str) -> dict:
    return {"value": r["value"], "unit": UNIT, "cores": procs, "kind": "port", "mode": mode,
            "sample": f"{CPU_KIND[mode]}: levels 0-{CPU_SAMPLE_LEVELS - 1} (whole searches) of {BEAMS} beams "
                      f"(seeds 0-{BEAMS - 1}), one process per beam, {r['busy']:.1f} s"}


def reference_arm(args) -> int:
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return 0
    procs = max(1, min(BEAMS, os.cpu_count() or 1))
    seeds = list(range(BEAMS))
    from oracle import oracle as O

    O.build(ref=False)
    vals, times = [], []
    with mp.get_context("spawn").Pool(procs) as pool:
        for _ in range(args.warmup):
            cpu_sample(procs, seeds, levels=20, pool=pool)
        # every step: whole 1 000-level searches of the 8 beams, whatever --steps is
        for _ in range(args.steps):
            r = cpu_sample(procs, seeds, levels=CPU_SAMPLE_LEVELS, pool=pool)
            vals.append(r["value"])
            times.append(r["busy"])
    value = sum(vals) / len(vals)
    sample = (f"{CPU_KIND['pms']}: whole {CPU_SAMPLE_LEVELS}-level searches of {BEAMS} beams (seeds 0-{BEAMS - 1}), "
              f"{procs} processes, per step")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * statistics.mean(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64",
            "data": "synthetic", "config": _config(world, "pms"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def _traffic(kernel: str):
    """DRAM bytes per launch of `kernel` on this workload, from the committed ncu summary
    (profiles/ncu_traffic.txt lines: kernel=<k> workload=<w> dram_bytes_per_launch=<x>)."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        kv = dict(tok.split("=", 1) for tok in line.split() if "=" in tok)
        if kv.get("kernel") == kernel and kv.get("workload") == f"{N_JOBS}x{N_MACH}_K{K}_B{BEAMS}":
            try:
                return float(kv["dram_bytes_per_launch"])
            except (KeyError, ValueError):
                return None
    return None


def replica_seeds(rank: int):
    """Search seeds of one replica's beams: rank r runs seeds 8r .. 8r+7, so the N replicas
    together run N*8 distinct seeds (the reference's MPI ranks, gpu/v1/main.cu:56-60)."""
    return [BEAMS * rank + b for b in range(BEAMS)]


def aggregate_replicas(t_local: float, units_local: float, dist, device: str):
    """Whole-job figures over the replicas: the slowest rank's time and the units of all
    ranks (value = units / time).  Without a process group the local figures."""
    if not dist:
        return float(t_local), float(units_local)
    import torch

    tt = torch.tensor([float(t_local)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    uu = torch.tensor([float(units_local)], dtype=torch.float64, device=device)
    dist.all_reduce(uu)
    return float(tt.item()), float(uu.item())


def gpu_arm(args) -> int:
    import numpy as np
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    cpu = cpu_pms = None
    if rank == 0 and not args.no_cpu_baseline:
        # oracle pool started (spawn) before this process touches the GPU
        procs = max(1, min(BEAMS, os.cpu_count() or 1))
        from oracle import oracle as O

        O.build(ref=False)
        with mp.get_context("spawn").Pool(procs) as pool:
            cpu = cpu_baseline_entry(cpu_sample(procs, list(range(BEAMS)), pool=pool, mode=MODE), procs, MODE)
            cpu_pms = cpu_baseline_entry(cpu_sample(procs, list(range(BEAMS)), pool=pool, mode="pms"), procs, "pms")

    torch.cuda.set_device(local)
    from beamsearch_jssp_gpu_gb300 import BeamSpec, Context, synthetic_instance

    mc, du = synthetic_instance(N_JOBS, N_MACH, INSTANCE_SEED)
    ctx = Context(local)
    beams = [BeamSpec(MODE, K, 500000, sd, 0, 0) for sd in replica_seeds(rank)]
    plan = ctx.plan([(mc, du)], beams)
    stream = torch.cuda.Stream()            # explicit stream: a handle of 0 would select the context's own
    sh = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    with torch.cuda.stream(stream):
        plan.set_timing(False)
        if args.step_form is None:
            # autotuner: k_step form for this shape (untimed; results do not depend on it)
            tune = plan.autotune(repeats=1, stream=sh)
        else:
            plan.chunk = args.step_form
            tune = {"chunk": args.step_form, "ms": {}}
        for _ in range(args.warmup):
            plan.run(sh)
        torch.cuda.synchronize()

        clocks = ClockSampler(local)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        clocks.start()
        times = []
        for _ in range(args.steps):
            flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.run(sh)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        clk = clocks.stop()
        stats = plan.stats()
        res = plan.results(with_sequence=False)
        # per-kernel device times: one more step of the same plan with CUDA events around
        # every launch (event nodes slow the graph, so they stay out of the timed steps)
        plan.set_timing(True)
        flush.fill_(1)
        plan.run(sh)
        torch.cuda.synchronize()
        kms = plan.kernel_ms()
    expanded = sum(r["expanded"] for r in res)
    launches_per_step = plan.launches
    t_step, expanded_all = aggregate_replicas(sum(times) / len(times), expanded, dist, "cuda")
    value = expanded_all / (t_step / 1000.0)

    # e2e: the C ABI from host buffers (instance upload + all levels + results/schedules back)
    e2e_times = []
    with torch.cuda.stream(stream):
        for k in range(args.warmup + args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = ctx.solve_batch([(mc, du)], beams, sh)
            t1 = time.perf_counter()
            if k >= args.warmup:
                e2e_times.append(t1 - t0)
            assert sum(r["expanded"] for r in out) == expanded
    e2e_t, _ = aggregate_replicas(sum(e2e_times) / len(e2e_times), 0, dist, "cuda")
    h2d = mc.nbytes + du.nbytes + 24 * BEAMS
    d2h = BEAMS * (N_JOBS * N_MACH * 4 + 48)

    # roofline of the dominant kernel (CUDA-event times of the profiled step)
    peaks = _peaks()
    alg = {"k_step": stats["step_bytes"], "k_select": stats["select_bytes"]}
    dom = max(("k_step", "k_select"), key=lambda k: kms[k][0])
    ms, nl = kms[dom]
    per_launch_bytes = alg[dom] / nl
    achieved = per_launch_bytes / (ms / nl / 1000.0) / 1e9
    traffic = _traffic(dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                "algorithmic_bytes_per_launch": per_launch_bytes, "avg_launch_us": 1000.0 * ms / nl,
                "peak_source": peaks["source"],
                "regime": "latency-bound: each level of a beam is a dependent chain (select on a 2- or 4-SM "
                          "cluster, then materialise+expand); the per-level set (~5 MB per beam) stays "
                          "L2-resident, so neither HBM bandwidth nor an SM pipe is saturated",
                "kernel_share": {k: v[0] / max(1e-9, sum(x[0] for x in kms.values())) for k, v in kms.items()}}

    extras = {}
    if rank == 0 and not args.no_extras:
        extras["pms_exact"] = pms_exact(ctx, mc, du, stream)
        extras["batched"] = batched_stream(ctx)
        extras["serving"] = served_stream(ctx, local)
        extras["serving_mixed_branching"] = served_mixed_branching(ctx, local)

    if rank == 0 and cpu:
        extras["cpu_baseline_pms"] = cpu_pms
        matched = {"value_over_cpu_baseline": value / cpu["value"],
                   "e2e_over_cpu_baseline": (expanded_all / e2e_t) / cpu["value"]}
        if "pms_exact" in extras:
            matched["pms_exact_over_cpu_baseline_pms"] = extras["pms_exact"]["expanded_per_s"] / cpu_pms["value"]
        extras["matched_ratios"] = matched
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "int32+f32", "data": "synthetic", "config": _config(world),
                "e2e": {"value": expanded_all / e2e_t, "unit": UNIT, "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "gpu_launches": launches_per_step * args.steps, "roofline": roofline,
                "cpu_baseline": cpu, "clocks": clk,
                "select_fallback_levels": stats["select_fallbacks"],
                "autotune": {"chunk": tune["chunk"], "ms_per_candidate": {str(k): round(v, 3) for k, v in
                                                                          tune["ms"].items()}},
                "makespans": [r["makespan"] for r in res], **extras}
        print(json.dumps(line), flush=True)
    plan.close()
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


# ------------------------------------------------------------------------------------
# BS-PMS exact mode, batched and served streams (rank 0, after the headline measurement)
# ------------------------------------------------------------------------------------
def pms_exact(ctx, mc, du, stream) -> dict:
    """The headline's 8 beams in BS-PMS mode (cpu/v1_pms/solver.cpp semantics: glibc rand()
    pivots and noise, fp64 score, libstdc++ bounded heap; makespans equal to the reference's
    CPU solver for the same srand seeds 0-7, which are the cpu_baseline's seeds).  The heap
    is serial per beam (k_heap), so this is one search per SM, not the throughput path."""
    import torch

    from beamsearch_jssp_gpu_gb300 import BeamSpec

    beams = [BeamSpec("pms", K, 500000, sd, 0, 0) for sd in range(BEAMS)]
    plan = ctx.plan([(mc, du)], beams)
    plan.run(stream.cuda_stream)
    plan.results(with_sequence=False)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    plan.run(stream.cuda_stream)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    res = plan.results(with_sequence=False)
    plan.close()
    expanded = sum(r["expanded"] for r in res)
    return {"workload": f"{BEAMS} beams, BS-PMS mode, {N_JOBS}x{N_MACH}, K={K}, srand seeds 0-{BEAMS - 1}",
            "expanded_per_s": expanded / (ms / 1000.0), "ms_per_search": ms,
            "makespans": [r["makespan"] for r in res]}


def batched_stream(ctx, count: int = 256, seed: int = 1) -> dict:
    """256 synthetic instances of uneven size in one set of launches (bsj_solve_batch),
    against the plain path: the same instances solved one call at a time (bsj_solve)."""
    import random

    from beamsearch_jssp_gpu_gb300 import BeamSpec, synthetic_instance

    rng = random.Random(seed)
    insts, beams = [], []
    for i in range(count):
        n = rng.choice([10, 15, 20, 30, 50, 100])
        m = rng.choice([5, 10, 15, 20])
        K = rng.choice([256, 512, 1024, 4096])
        insts.append(synthetic_instance(n, m, 10000 + i))
        beams.append(BeamSpec("v2", K, 500000, rng.randrange(1 << 30), i, -1))
    ctx.set_autotune(True)
    ctx.solve_batch(insts, beams)                      # builds, tunes and caches the batch plan
    ctx.set_autotune(False)
    t0 = time.perf_counter()
    out = ctx.solve_batch(insts, beams)
    t_batch = time.perf_counter() - t0
    t0 = time.perf_counter()
    plain = [ctx.solve(mc, du, b.mode, b.beam_width, b.seed) for (mc, du), b in zip(insts, beams)]
    t_plain = time.perf_counter() - t0
    same = all(a["makespan"] == b["makespan"] and a["expanded"] == b["expanded"] for a, b in zip(out, plain))
    return {"workload": f"{count} instances, n in {{10,15,20,30,50,100}}, m in {{5,10,15,20}}, "
                        f"K in {{256,512,1024,4096}}, gpu-v2 mode, one batch of launches",
            "solves_per_s": count / t_batch, "plain_solves_per_s": count / t_plain,
            "speedup_vs_plain": t_plain / t_batch, "identical_makespans": same,
            "expanded_per_s": sum(r["expanded"] for r in out) / t_batch}


def _serve(srv, reqs, rate: float, seed: int):
    """Open-loop Poisson arrivals of `reqs` at `rate`; returns the results in request order
    and the span from the first submission to the last result."""
    import numpy as np

    gaps = np.random.default_rng(seed).exponential(1.0 / rate, len(reqs))
    tickets = []
    t0 = time.perf_counter()
    arrival = t0
    for r, g in zip(reqs, gaps):
        arrival += g
        while time.perf_counter() < arrival:
            pass
        tickets.append(srv.submit(*r))
    got = [srv.wait(t) for t in tickets]
    return got, time.perf_counter() - t0


def _plain(ctx, reqs):
    """The plain path: every request solved alone, one call at a time (bsj_solve); returns
    the results, each request's own solve time (ms) and the total seconds."""
    out, ms = [], []
    t0 = time.perf_counter()
    for r in reqs:
        t1 = time.perf_counter()
        out.append(ctx.solve(*r))
        ms.append(1000.0 * (time.perf_counter() - t1))
    return out, ms, time.perf_counter() - t0


def _latency(got, solo_ms=None) -> dict:
    """p50/p99 of queue + run time, over all requests and split by whether the request found
    an idle plan of its shape or built one; with `solo_ms` (each request's time solved alone)
    also the stretch, latency / solo time, which removes the spread of search lengths in the
    mix (a 100x20 K=4096 search takes ~30x a 15x15 K=256 one)."""
    import numpy as np

    out = {}
    if solo_ms is not None:
        st = np.array([(g["queue_ms"] + g["run_ms"]) / max(1e-3, t) for g, t in zip(got, solo_ms)])
        out["stretch"] = {"p50": float(np.percentile(st, 50)), "p99": float(np.percentile(st, 99))}
    for name, sel in (("all", lambda g: True), ("reused_plan", lambda g: not g["built_plan"]),
                      ("built_plan", lambda g: g["built_plan"])):
        lat = np.array([g["queue_ms"] + g["run_ms"] for g in got if sel(g)])
        out[name] = ({"count": int(lat.size), "p50_ms": float(np.percentile(lat, 50)),
                      "p99_ms": float(np.percentile(lat, 99))} if lat.size else {"count": 0})
    return out


def _warm(srv, reqs, copies: int):
    """Before traffic: `copies` prepared plans of every request shape (bsj_server_prepare),
    as a long-running server holds for the shapes it serves."""
    shapes = {}
    for r in reqs:
        shapes.setdefault((r[0].shape, r[2], r[3]), r)
    for r in shapes.values():
        srv.prepare(r[0], r[1], r[2], r[3], copies=copies, seed=r[4])
    deadline = time.time() + 600
    while srv.stats()["plans_prepared"] < copies * len(shapes):
        if time.time() > deadline:
            raise RuntimeError("prepared plans not ready within 10 minutes")
        time.sleep(0.01)
    return len(shapes)


def served_stream(ctx, device: int, count: int = 400, rates=(150.0, 1000.0), inflight: int = 96,
                  seed: int = 5, warm_copies: int = 8) -> dict:
    """Open-loop Poisson arrivals served by bsj_server (continuous batching), at a rate the
    server sustains and at one it cannot (queueing), against the plain path solving the same
    requests one at a time.  Every result is compared with the plain path's.  Before the
    timed streams the server prepares `warm_copies` plans of every request shape; latency is
    reported over all requests and split by requests that reused a plan / built one."""
    import random

    import numpy as np

    from beamsearch_jssp_gpu_gb300 import Server, synthetic_instance

    rng = random.Random(seed)
    reqs = []
    for i in range(count):
        n = rng.choice([15, 20, 30, 50, 100])
        m = rng.choice([15, 20])
        K = rng.choice([256, 1024, 4096])
        mode = rng.choice(["v2", "clean"])
        mc, du = synthetic_instance(n, m, 20000 + i)
        reqs.append((mc, du, mode, K, rng.randrange(1 << 30)))
    plain, solo_ms, t_plain = _plain(ctx, reqs)
    runs = []
    same = True
    with Server(device, max_inflight=inflight) as srv:
        nshapes = _warm(srv, reqs, warm_copies)
        for rate in rates:
            got, span = _serve(srv, reqs, rate, seed)
            same = same and all(a["makespan"] == b["makespan"] and np.array_equal(a["seq"], b["seq"])
                                for a, b in zip(plain, got))
            lat = _latency(got, solo_ms)
            runs.append({"offered_per_s": rate, "solves_per_s": count / span, "p50_ms": lat["all"]["p50_ms"],
                         "p99_ms": lat["all"]["p99_ms"], "latency": lat})
        st = srv.stats()
    best = max(runs, key=lambda x: x["solves_per_s"])
    return {"workload": f"{count} requests per rate, Poisson arrivals, n in {{15,20,30,50,100}}, m in "
                        f"{{15,20}}, K in {{256,1024,4096}}, gpu-v2/clean modes, {inflight} slots, "
                        f"{warm_copies} prepared plans per shape ({nshapes} shapes)",
            "solves_per_s": best["solves_per_s"], "p50_ms": best["p50_ms"], "p99_ms": best["p99_ms"],
            "rates": runs, "plain_solves_per_s": count / t_plain,
            "speedup_vs_plain": best["solves_per_s"] / (count / t_plain), "identical_results": same,
            "plans_built": st["plans_built"], "plans_prepared": st["plans_prepared"],
            "plans_reused": st["plans_reused"], "peak_inflight": st["peak_inflight"]}


def served_mixed_branching(ctx, device: int, count: int = 96, rate: float = 40.0, inflight: int = 96,
                           seed: int = 7) -> dict:
    """The served stream with mixed ICH/PMS branching: half the requests are BS-ICH / BS-PMS
    (the CPU solvers' exact semantics: every ready op or the pivot machine's ops branched,
    glibc rand(), serial bounded heap per request) at K=256, half gpu-v2 / clean at K in
    {256, 1024, 4096}; n in {15, 20, 30, 50, 100}, m in {15, 20}.  The exact-semantics
    requests stay at K=256 so that the plain one-at-a-time comparison finishes within the
    bench's minutes (their heap is serial: a K=4096 100x20 BS-ICH search alone takes
    seconds).  Plans are prepared for every shape first; results are compared with the
    plain path."""
    import random

    import numpy as np

    from beamsearch_jssp_gpu_gb300 import Server, synthetic_instance

    rng = random.Random(seed)
    reqs = []
    for i in range(count):
        n = rng.choice([15, 20, 30, 50, 100])
        m = rng.choice([15, 20])
        mode = rng.choice(["ich", "pms", "v2", "clean"])
        K = 256 if mode in ("ich", "pms") else rng.choice([256, 1024, 4096])
        mc, du = synthetic_instance(n, m, 30000 + i)
        reqs.append((mc, du, mode, K, rng.randrange(1 << 30)))
    plain, solo_ms, t_plain = _plain(ctx, reqs)
    with Server(device, max_inflight=inflight) as srv:
        nshapes = _warm(srv, reqs, 2)
        got, span = _serve(srv, reqs, rate, seed)
        st = srv.stats()
    same = all(a["makespan"] == b["makespan"] and np.array_equal(a["seq"], b["seq"]) for a, b in zip(plain, got))
    lat = _latency(got, solo_ms)
    by_mode = {}
    for md in ("ich", "pms", "v2", "clean"):
        sel = [g for g, r in zip(got, reqs) if r[2] == md]
        if sel:
            x = np.array([g["queue_ms"] + g["run_ms"] for g in sel])
            by_mode[md] = {"count": len(sel), "p50_ms": float(np.percentile(x, 50)),
                           "p99_ms": float(np.percentile(x, 99))}
    return {"workload": f"{count} requests, Poisson {rate:g}/s, ICH/PMS at K=256 and gpu-v2/clean at K in "
                        f"{{256,1024,4096}}, n in {{15,20,30,50,100}}, m in {{15,20}}, {inflight} slots, "
                        f"2 prepared plans per shape ({nshapes} shapes)",
            "offered_per_s": rate, "solves_per_s": count / span, "p50_ms": lat["all"]["p50_ms"],
            "p99_ms": lat["all"]["p99_ms"], "latency": lat, "by_mode": by_mode,
            "plain_solves_per_s": count / t_plain, "speedup_vs_plain": t_plain / span,
            "identical_results": same, "plans_built": st["plans_built"], "plans_reused": st["plans_reused"]}


def k_sweep(args) -> int:
    """Time vs beam width on the GPU path (the GPU analogue of cpu/profiling/
    time_width_study.cpp): 20x15 synthetic instance, gpu-v1 mode, K in {256, 1024, 4096,
    16384}; per K one beam alone and the four seeds 0-3 as four beams of one launch.
    One JSON line per (K, beams): ms per search, us per level, expanded candidates/s and
    the algorithmic bytes per level over the level time."""
    import torch

    from beamsearch_jssp_gpu_gb300 import BeamSpec, Context, synthetic_instance

    n, m = 20, 15
    mc, du = synthetic_instance(n, m, 0)
    ctx = Context(0)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    peaks = _peaks()
    for K in (256, 1024, 4096, 16384):
        for nb in (1, 4):
            plan = ctx.plan([(mc, du)], [BeamSpec("v1", K, 500000, b, 0, -1) for b in range(nb)])
            with torch.cuda.stream(stream):
                for _ in range(args.warmup):
                    plan.run(sh)
                times = []
                for _ in range(args.steps):
                    flush.fill_(1)
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    plan.run(sh)
                    e1.record(stream)
                    e1.synchronize()
                    times.append(e0.elapsed_time(e1))
                st = plan.stats()
                res = plan.results(with_sequence=False)
            t = statistics.median(times)
            levels = n * m
            alg = st["step_bytes"] + st["select_bytes"]
            print(json.dumps({"metric": "k-sweep, 20x15, gpu-v1", "beam_width": K, "beams": nb,
                              "ms_per_search": t, "us_per_level": 1000.0 * t / levels,
                              "expanded_per_s": st["expanded"] / (t / 1000.0),
                              "alg_bytes_per_level": alg / levels,
                              "alg_gbs": alg / (t / 1000.0) / 1e9,
                              "hbm_frac": alg / (t / 1000.0) / 1e9 / peaks["hbm_gbs"],
                              "makespans": [r["makespan"] for r in res]}), flush=True)
            plan.close()
    ctx.close()
    return 0


def chunk_sweep(args) -> int:
    """Autotuner data: per shape (n, m, K, beams; gpu-v2 mode) the ms per search of each
    k_step chunk candidate (0 = the default rule; 8, 16, 32 survivors per thread block),
    from bsj_plan_autotune.  One JSON line per shape."""
    import torch

    from beamsearch_jssp_gpu_gb300 import BeamSpec, Context, synthetic_instance

    shapes = [(10, 5, 256, 1), (15, 15, 256, 1), (20, 15, 256, 1), (20, 15, 1024, 1), (20, 15, 1024, 8),
              (20, 15, 4096, 1), (20, 15, 4096, 8), (30, 20, 1024, 1), (30, 20, 4096, 1), (30, 20, 4096, 8),
              (50, 20, 256, 1), (50, 20, 1024, 1), (50, 20, 4096, 1), (50, 20, 4096, 8), (100, 20, 1024, 1),
              (100, 20, 4096, 1), (100, 20, 4096, 8), (20, 15, 16384, 1)]
    ctx = Context(0)
    stream = torch.cuda.Stream()
    for n, m, K, nb in shapes:
        mc, du = synthetic_instance(n, m, 0)
        plan = ctx.plan([(mc, du)], [BeamSpec("v2", K, 500000, b, 0, 0) for b in range(nb)])
        with torch.cuda.stream(stream):
            out = plan.autotune(repeats=max(1, args.steps), stream=stream.cuda_stream)
        print(json.dumps({"metric": "chunk-sweep, gpu-v2", "jobs": n, "machines": m, "beam_width": K,
                          "beams": nb, "chunk": out["chunk"],
                          "ms": {str(c): round(v, 3) for c, v in out["ms"].items()}}), flush=True)
        plan.close()
    ctx.close()
    return 0


def solve_times(args) -> int:
    """Single searches on the GPU path, one beam per plan (default chunk rule), in the gpu
    modes: 20x15 K=1024 and 50x20 K=4096, synthetic instance seed 0, search seed 0 -- the
    cases the reference's own gpu kernels are timed on by the oracle's timing script.
    CUDA events on an explicit stream, median of `--steps` runs after `--warmup`."""
    import torch

    from beamsearch_jssp_gpu_gb300 import BeamSpec, Context, synthetic_instance

    ctx = Context(0)
    stream = torch.cuda.Stream()
    for n, m, K in ((20, 15, 1024), (50, 20, 4096)):
        mc, du = synthetic_instance(n, m, 0)
        for mode in ("v2", "v1"):
            plan = ctx.plan([(mc, du)], [BeamSpec(mode, K, 500000, 0, 0, -1)])
            with torch.cuda.stream(stream):
                for _ in range(args.warmup):
                    plan.run(stream.cuda_stream)
                times = []
                for _ in range(args.steps):
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    plan.run(stream.cuda_stream)
                    e1.record(stream)
                    e1.synchronize()
                    times.append(e0.elapsed_time(e1))
            r = plan.results(with_sequence=False)[0]
            print(json.dumps({"solver": f"engine {mode}", "jobs": n, "machines": m, "beam_width": K, "seed": 0,
                              "ms_per_search": statistics.median(times), "makespan": r["makespan"]}), flush=True)
            plan.close()
    ctx.close()
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched and served streams")
    ap.add_argument("--k-sweep", action="store_true", help="time vs beam width (20x15, gpu-v1), one line per K")
    ap.add_argument("--chunk-sweep", action="store_true",
                    help="ms per search of each k_step chunk size over a set of shapes (autotuner data)")
    ap.add_argument("--step-form", type=int, default=None, choices=[0, 8, 16, 32, 1, 2, 3, 4],
                    help="run the headline plan with this k_step form (0 = default rule; 8/16/32 warp per "
                         "survivor; 1-4 lane group per survivor) instead of autotuning it")
    ap.add_argument("--solve-times", action="store_true",
                    help="single gpu-v1/v2 searches (20x15 K=1024, 50x20 K=4096): ms per search")
    args = ap.parse_args()
    if args.solve_times:
        return solve_times(args)
    if args.k_sweep:
        return k_sweep(args)
    if args.chunk_sweep:
        return chunk_sweep(args)
    if args.impl == "reference":
        return reference_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
