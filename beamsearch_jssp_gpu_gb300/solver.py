"""Python front end of the solver library, mirroring the reference's entry points.

``run_gpu_beam_search_v1`` / ``run_gpu_beam_search_v2`` keep the reference's names,
argument meaning and return value (gpu/v1/solver.cuh:6-12, gpu/v2_twophases/solver.cuh:
6-12); ``beam_search_ich`` / ``beam_search_pms`` are the GPU forms of the CPU solvers
(cpu/v0_ich/solver.h:6, cpu/v1_pms/solver.h:6) with the ``srand`` seed made explicit.
Everything runs through libbsj.so's C ABI on the GPU; errors raise ``BsjError``.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import _native as nat
from .instance import JSSPInstance

__all__ = ["Context", "Plan", "BeamSpec", "run_gpu_beam_search_v1", "run_gpu_beam_search_v2",
           "beam_search_ich", "beam_search_pms", "solve", "solve_batch", "solve_iterations", "Server"]


def _i32p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


@dataclass
class BeamSpec:
    """One beam of a batch (include/bsj.h ``bsj_beam``)."""

    mode: str = "v2"
    beam_width: int = 1024
    best_known: int = nat.NO_BOUND
    seed: int = 0
    instance: int = 0
    bound_group: int = -1

    def to_c(self) -> nat.Beam:
        if self.mode not in nat.MODES:
            raise ValueError(f"unknown mode {self.mode!r}; one of {sorted(nat.MODES)}")
        return nat.Beam(nat.MODES[self.mode], int(self.beam_width), int(self.best_known),
                        int(self.seed) & 0xFFFFFFFF, int(self.instance), int(self.bound_group))


class _InstanceArrays:
    """Keeps the int32 arrays of a batch of instances alive for a C call."""

    def __init__(self, instances):
        self.arrays = []
        self.c = (nat.Instance * len(instances))()
        for k, inst in enumerate(instances):
            if isinstance(inst, JSSPInstance):
                mc, du = inst.machine, inst.duration
            else:
                mc, du = inst
            mc = np.ascontiguousarray(mc, dtype=np.int32)
            du = np.ascontiguousarray(du, dtype=np.int32)
            if mc.ndim != 2 or mc.shape != du.shape:
                raise ValueError("an instance is a pair of [n, m] int arrays (machine, duration)")
            self.arrays.append((mc, du))
            self.c[k] = nat.Instance(mc.shape[0], mc.shape[1], _i32p(mc), _i32p(du))
        self.sizes = [a[0].shape for a in self.arrays]


class Context:
    """A solver context on one CUDA device (``bsj_create``)."""

    def __init__(self, device: int = -1):
        self.lib = nat.load()
        h = ctypes.c_void_p()
        st = self.lib.bsj_create(ctypes.byref(h), int(device))
        if st != nat.BSJ_OK:
            raise nat.BsjError(st, f"bsj_create(device={device}) failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.bsj_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int):
        if st != nat.BSJ_OK:
            raise nat.BsjError(st, self.lib.bsj_last_error(self.h).decode(errors="replace"))

    def solve_batch(self, instances: Sequence, beams: Sequence[BeamSpec], stream: int = 0) -> List[dict]:
        ia = _InstanceArrays(instances)
        cb = (nat.Beam * len(beams))(*[b.to_c() for b in beams])
        res = (nat.Result * len(beams))()
        seqs = []
        for k, b in enumerate(beams):
            n, m = ia.sizes[b.instance] if 0 <= b.instance < len(ia.sizes) else (0, 0)
            s = np.zeros(max(n * m, 1), dtype=np.int32)
            seqs.append(s)
            res[k].sequence = _i32p(s)
        st = self.lib.bsj_solve_batch(self.h, len(ia.arrays), ia.c, len(beams), cb, res,
                                      ctypes.c_void_p(stream) if stream else None)
        self._check(st)
        return [_result_dict(res[k], seqs[k]) for k in range(len(beams))]

    def solve(self, machine, duration, mode: str = "v2", beam_width: int = 1024, seed: int = 0,
              best_known: int = nat.NO_BOUND, stream: int = 0) -> dict:
        return self.solve_batch([(machine, duration)],
                                [BeamSpec(mode, beam_width, best_known, seed, 0, -1)], stream)[0]

    def solve_iterations(self, machine, duration, mode: str, beam_width: int, seeds,
                         initial_bound: int = nat.NO_BOUND, stream: int = 0, iterations: int = 0):
        """Multi-start passes with the bound carried between rounds (bsj_solve_iterations).

        Gpu modes: ``seeds`` is ``[iterations, beams]`` random_seeds.  ICH/PMS: ``seeds``
        is ``[beams]`` srand() seeds whose rand() streams run on across ``iterations``
        rounds.  Returns (best makespan, best sequence, best after each round)."""
        ia = _InstanceArrays([(machine, duration)])
        sd = np.ascontiguousarray(np.asarray(seeds, dtype=np.int64) & 0xFFFFFFFF, dtype=np.uint32)
        carry = nat.MODES[mode] >= nat.MODES["ich"]
        if carry:
            if sd.ndim != 1 or iterations < 1:
                raise ValueError("ICH/PMS: seeds must be [beams] and iterations >= 1")
            beams, rounds = sd.shape[0], int(iterations)
        else:
            if sd.ndim != 2:
                raise ValueError("seeds must be [iterations, beams]")
            rounds, beams = sd.shape
        best = ctypes.c_int32()
        n, m = ia.sizes[0]
        seq = np.zeros(n * m, dtype=np.int32)
        per_round = np.zeros(rounds, dtype=np.int32)
        st = self.lib.bsj_solve_iterations(self.h, ia.c, nat.MODES[mode], int(beam_width), beams, rounds,
                                           sd.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                           int(initial_bound), ctypes.byref(best), _i32p(seq), _i32p(per_round),
                                           ctypes.c_void_p(stream) if stream else None)
        self._check(st)
        return best.value, seq, per_round

    def plan(self, instances: Sequence, beams: Sequence[BeamSpec]) -> "Plan":
        return Plan(self, instances, beams)

    def set_autotune(self, on: bool):
        """Tune every new batch shape on its first solve (bsj_set_autotune)."""
        self._check(self.lib.bsj_set_autotune(self.h, 1 if on else 0))

    def estimate(self, instances: Sequence, beams: Sequence[BeamSpec]) -> int:
        """Device bytes a plan of this batch would hold (bsj_plan_estimate)."""
        ia = _InstanceArrays(instances)
        cb = (nat.Beam * len(beams))(*[b.to_c() for b in beams])
        out = ctypes.c_int64()
        self._check(self.lib.bsj_plan_estimate(self.h, len(ia.arrays), ia.c, len(beams), cb, ctypes.byref(out)))
        return int(out.value)


class Plan:
    """A prepared batch (``bsj_plan_*``): inputs uploaded once, runs enqueued on a stream."""

    def __init__(self, ctx: Context, instances: Sequence, beams: Sequence[BeamSpec]):
        self.ctx = ctx
        self.lib = ctx.lib
        self._ia = _InstanceArrays(instances)
        self.beams = list(beams)
        cb = (nat.Beam * len(beams))(*[b.to_c() for b in beams])
        h = ctypes.c_void_p()
        ctx._check(self.lib.bsj_plan_create(ctx.h, len(self._ia.arrays), self._ia.c, len(beams), cb,
                                            ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.bsj_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, stream: int = 0):
        self.ctx._check(self.lib.bsj_plan_run(self.h, ctypes.c_void_p(stream) if stream else None))

    def results(self, with_sequence: bool = True) -> List[dict]:
        res = (nat.Result * len(self.beams))()
        seqs = []
        for k, b in enumerate(self.beams):
            n, m = self._ia.sizes[b.instance]
            s = np.zeros(n * m, dtype=np.int32)
            seqs.append(s)
            if with_sequence:
                res[k].sequence = _i32p(s)
        self.ctx._check(self.lib.bsj_plan_results(self.h, res))
        return [_result_dict(res[k], seqs[k] if with_sequence else None) for k in range(len(self.beams))]

    @property
    def launches(self) -> int:
        return int(self.lib.bsj_plan_launches(self.h))

    def stats(self):
        """Algorithmic bytes per kernel class of the last run, expanded children and
        materialised survivors (include/bsj.h bsj_plan_stats)."""
        sb = ctypes.c_double()
        selb = ctypes.c_double()
        e = ctypes.c_int64()
        mat = ctypes.c_int64()
        fb = ctypes.c_int64()
        self.ctx._check(self.lib.bsj_plan_stats(self.h, ctypes.byref(sb), ctypes.byref(selb), ctypes.byref(e),
                                                ctypes.byref(mat), ctypes.byref(fb)))
        return dict(step_bytes=sb.value, select_bytes=selb.value, expanded=e.value, materialized=mat.value,
                    select_fallbacks=fb.value)

    def set_timing(self, on: bool):
        self.ctx._check(self.lib.bsj_plan_set_timing(self.h, 1 if on else 0))

    def set_select_route(self, *flags: str):
        """Force the gpu-mode levels' top-K selection onto routes (names of
        ``_native.SELECT``: force_large, no_large, no_direct, radix, no_dense, rank_lsd,
        bitonic, no_cluster, force_cluster); no names = the normal choice by level size
        (bsj_plan_set_select_route)."""
        v = 0
        for f in flags:
            v |= nat.SELECT[f]
        self.ctx._check(self.lib.bsj_plan_set_select_route(self.h, v))

    def set_select_cluster(self, on: bool):
        """Cluster select where the rule picks it (True, the default) or one thread block per
        beam (False) from the next run on (bsj_plan_set_select_cluster); results unchanged."""
        self.ctx._check(self.lib.bsj_plan_set_select_cluster(self.h, 1 if on else 0))

    def select_routes(self) -> set:
        """Names (``_native.ROUTE``) of the selection routes the last run took."""
        r = ctypes.c_uint32()
        self.ctx._check(self.lib.bsj_plan_select_routes(self.h, ctypes.byref(r)))
        return {k for k, bit in nat.ROUTE.items() if r.value & bit}

    def autotune(self, repeats: int = 2, stream: int = 0) -> dict:
        """Time every k_step chunk candidate on this plan and keep the fastest
        (bsj_plan_autotune).  Returns {"chunk": choice, "ms": {candidate: ms per run}},
        candidates 0 (the default rule), 8, 16, 32."""
        ch = ctypes.c_int32()
        ms = (ctypes.c_float * len(nat.CHUNK_CANDIDATES))()
        self.ctx._check(self.lib.bsj_plan_autotune(self.h, ctypes.c_void_p(stream) if stream else None,
                                                   int(repeats), ctypes.byref(ch), ms))
        return {"chunk": int(ch.value), "ms": {c: float(ms[i]) for i, c in enumerate(nat.CHUNK_CANDIDATES)}}

    @property
    def chunk(self) -> int:
        """Survivors per k_step thread block: 8, 16 or 32 for every beam group, or 0 for
        the default rule's per-group sizes."""
        return int(self.lib.bsj_plan_chunk(self.h))

    @chunk.setter
    def chunk(self, value: int):
        self.ctx._check(self.lib.bsj_plan_set_chunk(self.h, int(value)))

    KERNELS = ("k_step", "k_select", "k_heap", "k_gather_v1", "k_finalize")

    def kernel_ms(self) -> dict:
        ms = (ctypes.c_float * 5)()
        cnt = (ctypes.c_int64 * 5)()
        self.ctx._check(self.lib.bsj_plan_kernel_ms(self.h, ms, cnt, 5))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.KERNELS)}


class Server:
    """Continuous-batching request loop on one GPU (include/bsj.h ``bsj_server_*``).

    ``submit`` queues one solve and returns a ticket at once; the server admits queued
    requests while an in-flight slot and the memory budget allow, runs them concurrently
    and reuses plans by shape.  ``poll`` / ``wait`` return the result dict with
    ``queue_ms`` and ``run_ms``.  Thread-safe.  ``cluster_inflight``: a request runs the
    cluster select (K >= 4096) only when at most this many others are in flight at its
    admission (0 = the device's SMs / 8, negative = never)."""

    def __init__(self, device: int = 0, max_inflight: int = 0, memory_budget: int = 0, cluster_inflight: int = 0):
        self.lib = nat.load()
        h = ctypes.c_void_p()
        cfg = nat.ServerConfig(int(max_inflight), int(cluster_inflight), int(memory_budget))
        st = self.lib.bsj_server_create(ctypes.byref(h), int(device), ctypes.byref(cfg))
        if st != nat.BSJ_OK:
            raise nat.BsjError(st, "cannot create the server")
        self.h = h
        self._n = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.bsj_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, machine, duration, mode: str = "v2", beam_width: int = 1024, seed: int = 0,
               best_known: int = nat.NO_BOUND) -> int:
        mc = np.ascontiguousarray(machine, dtype=np.int32)
        du = np.ascontiguousarray(duration, dtype=np.int32)
        n, m = mc.shape
        inst = nat.Instance(n, m, _i32p(mc), _i32p(du))
        beam = BeamSpec(mode, beam_width, best_known, seed).to_c()
        t = ctypes.c_uint64()
        st = self.lib.bsj_submit(self.h, ctypes.byref(inst), ctypes.byref(beam), ctypes.byref(t))
        if st != nat.BSJ_OK:
            raise nat.BsjError(st, "request rejected")
        self._n[t.value] = n * m
        return t.value

    def _finish(self, ticket, st, res, seq, times) -> dict:
        self._n.pop(ticket, None)
        if st != nat.BSJ_OK:
            raise nat.BsjError(st, f"request {ticket} failed")
        d = _result_dict(res, seq)
        d["queue_ms"] = times.queue_ms
        d["run_ms"] = times.run_ms
        d["built_plan"] = bool(times.built_plan)
        return d

    def prepare(self, machine, duration, mode: str = "v2", beam_width: int = 1024, copies: int = 1,
                seed: int = 0):
        """Build ``copies`` plans of this request shape (n, m, mode, K) ahead of traffic
        (bsj_server_prepare): later requests of the shape reuse them."""
        mc = np.ascontiguousarray(machine, dtype=np.int32)
        du = np.ascontiguousarray(duration, dtype=np.int32)
        n, m = mc.shape
        inst = nat.Instance(n, m, _i32p(mc), _i32p(du))
        beam = BeamSpec(mode, beam_width, nat.NO_BOUND, seed).to_c()
        st = self.lib.bsj_server_prepare(self.h, ctypes.byref(inst), ctypes.byref(beam), int(copies))
        if st != nat.BSJ_OK:
            raise nat.BsjError(st, "prepare rejected")

    def poll(self, ticket: int) -> Optional[dict]:
        seq = np.zeros(self._n.get(ticket, 1), dtype=np.int32)
        res = nat.Result()
        res.sequence = _i32p(seq)
        times = nat.RequestTimes()
        done = ctypes.c_int32()
        st = self.lib.bsj_poll(self.h, ctypes.c_uint64(ticket), ctypes.byref(res), ctypes.byref(times),
                               ctypes.byref(done))
        if st == nat.BSJ_OK and not done.value:
            return None
        return self._finish(ticket, st, res, seq, times)

    def wait(self, ticket: int) -> dict:
        seq = np.zeros(self._n.get(ticket, 1), dtype=np.int32)
        res = nat.Result()
        res.sequence = _i32p(seq)
        times = nat.RequestTimes()
        st = self.lib.bsj_wait(self.h, ctypes.c_uint64(ticket), ctypes.byref(res), ctypes.byref(times))
        return self._finish(ticket, st, res, seq, times)

    def stats(self) -> dict:
        s = nat.ServerStats()
        st = self.lib.bsj_server_get_stats(self.h, ctypes.byref(s))
        if st != nat.BSJ_OK:
            raise nat.BsjError(st, "stats")
        return {k: (float if t is ctypes.c_double else int)(getattr(s, k)) for k, t in nat.ServerStats._fields_}


def _result_dict(r: nat.Result, seq) -> dict:
    return dict(makespan=int(r.makespan), found=bool(r.found), seq=seq, expanded=int(r.expanded),
                slots=int(r.slots), levels=int(r.levels), group_best=int(r.group_best))


_default_ctx: Optional[Context] = None


def _ctx() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(-1)
    return _default_ctx


def solve(machine, duration, mode="v2", beam_width=1024, seed=0, best_known=nat.NO_BOUND) -> dict:
    return _ctx().solve(machine, duration, mode, beam_width, seed, best_known)


def solve_batch(instances, beams) -> List[dict]:
    return _ctx().solve_batch(instances, beams)


def solve_iterations(machine, duration, mode, beam_width, seeds, initial_bound=nat.NO_BOUND, iterations=0):
    return _ctx().solve_iterations(machine, duration, mode, beam_width, seeds, initial_bound,
                                   iterations=iterations)


def _run_ref_style(mode: str, inst: JSSPInstance, beam_width: int, best_known: int, random_seed: int,
                   out_best_sequence) -> int:
    r = _ctx().solve(inst.machine, inst.duration, mode, beam_width, random_seed, best_known)
    if out_best_sequence is not None and r["makespan"] < nat.NO_BOUND:
        out_best_sequence[: len(r["seq"])] = r["seq"]
    return r["makespan"]


def run_gpu_beam_search_v1(inst: JSSPInstance, beam_width: int, best_known: int, random_seed: int,
                           out_best_sequence=None) -> int:
    """gpu/v1/solver.cuh:6-12: returns min(best_known, best complete makespan) and fills
    ``out_best_sequence`` (a mutable sequence of >= n*m ints) when the result < 500000."""
    return _run_ref_style("v1", inst, beam_width, best_known, random_seed, out_best_sequence)


def run_gpu_beam_search_v2(inst: JSSPInstance, beam_width: int, best_known: int, random_seed: int,
                           out_best_sequence=None) -> int:
    """gpu/v2_twophases/solver.cuh:6-12, same contract as run_gpu_beam_search_v1."""
    return _run_ref_style("v2", inst, beam_width, best_known, random_seed, out_best_sequence)


def beam_search_ich(inst: JSSPInstance, beam_width: int, seed: int = 12345) -> int:
    """cpu/v0_ich/solver.cpp:8-54 on the GPU, after ``srand(seed)`` (12345 in
    cpu/v0_ich/main.cpp:39)."""
    return _ctx().solve(inst.machine, inst.duration, "ich", beam_width, seed)["makespan"]


def beam_search_pms(inst: JSSPInstance, beam_width: int, best_known: int, seed: int) -> int:
    """cpu/v1_pms/solver.cpp:8-70 on the GPU, after ``srand(seed)``."""
    return _ctx().solve(inst.machine, inst.duration, "pms", beam_width, seed, best_known)["makespan"]
