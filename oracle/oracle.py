"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py as the
checker.  The product package never imports this module.

``liborc.so`` is the C restatement in bsj_oracle.c (built by ``build()`` here and on the
GPU machine); ``_ref/libref_cpu.so`` is the reference's own CPU solvers compiled from
their sources, present only where the reference tree is (this container).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORC_LIB = os.path.join(HERE, "_build", "liborc.so")
REF_CPU_LIB = os.path.join(HERE, "_ref", "libref_cpu.so")

MODES = {"v1": 0, "v2": 1, "clean": 2, "ich": 3, "pms": 4}
MARK = 0xFFFFFFFF


class _Instance(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int),
        ("m", ctypes.c_int),
        ("machine", ctypes.POINTER(ctypes.c_int32)),
        ("duration", ctypes.POINTER(ctypes.c_int32)),
    ]


class _Params(ctypes.Structure):
    _fields_ = [
        ("mode", ctypes.c_int),
        ("beam_width", ctypes.c_int),
        ("best_known", ctypes.c_int),
        ("seed", ctypes.c_uint32),
        ("trace", ctypes.POINTER(ctypes.c_uint32)),
        ("trace_count", ctypes.POINTER(ctypes.c_int32)),
        ("ties", ctypes.POINTER(ctypes.c_int32)),
        ("max_ties", ctypes.c_int32),
    ]


class _Result(ctypes.Structure):
    _fields_ = [
        ("makespan", ctypes.c_int32),
        ("found", ctypes.c_int32),
        ("seq", ctypes.POINTER(ctypes.c_int32)),
        ("expanded", ctypes.c_int64),
        ("slots", ctypes.c_int64),
        ("levels", ctypes.c_int32),
        ("ties", ctypes.c_int32),
    ]


def build(ref: Optional[bool] = None) -> None:
    """Compile liborc.so; also the reference's own solvers from their sources: with
    ``ref=None`` when the reference tree exists (``make ref-if-present``; the tree's
    location is the Makefile's, overridable by BSJ_REFERENCE_TREE), with ``ref=True``
    always (``make ref``)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    if ref is None:
        subprocess.check_call(["make", "-s", "-C", HERE, "ref-if-present"])
    elif ref:
        subprocess.check_call(["make", "-s", "-C", HERE, "ref"])


def reference_tree() -> str:
    """Location of the reference tree as the Makefile resolves it (BSJ_REFERENCE_TREE, else
    the recipe's default); the tree may be absent."""
    return subprocess.check_output(["make", "-s", "--no-print-directory", "-C", HERE, "print-ref"],
                                   text=True).strip()


_orc = None


def _lib():
    global _orc
    if _orc is None:
        if not os.path.exists(ORC_LIB):
            build(ref=False)
        lib = ctypes.CDLL(ORC_LIB)
        lib.orc_solve_levels.argtypes = [
            ctypes.POINTER(_Instance),
            ctypes.POINTER(_Params),
            ctypes.POINTER(_Result),
            ctypes.c_int,
        ]
        lib.orc_solve_levels.restype = ctypes.c_int
        lib.orc_glibc_rand_fill.argtypes = [ctypes.c_uint32, ctypes.POINTER(ctypes.c_int32), ctypes.c_int]
        lib.orc_pivot_hash.argtypes = [ctypes.c_uint32]
        lib.orc_pivot_hash.restype = ctypes.c_uint32
        lib.orc_noise_hash.argtypes = [ctypes.c_uint32] * 3
        lib.orc_noise_hash.restype = ctypes.c_uint32
        lib.orc_gpu_score.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]
        lib.orc_gpu_score.restype = ctypes.c_float
        lib.orc_schedule_makespan.argtypes = [ctypes.POINTER(_Instance), ctypes.POINTER(ctypes.c_int32)]
        lib.orc_schedule_makespan.restype = ctypes.c_int32
        lib.orc_solve_iterations.argtypes = [
            ctypes.POINTER(_Instance), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
            ctypes.POINTER(ctypes.c_uint32), ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
            ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
        lib.orc_solve_iterations.restype = ctypes.c_int
        _orc = lib
    return _orc


def _ptr(a: np.ndarray):
    ctype = ctypes.c_uint32 if a.dtype == np.uint32 else ctypes.c_int32
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def solve(machine, duration, mode: str, K: int, seed: int, best_known: int = 500000,
          trace: bool = False, max_levels: int = 1 << 30, max_ties: int = 0) -> dict:
    """Run the oracle; returns makespan, found, seq (1-based op ids), expanded, slots,
    levels, ties; with ``trace`` the per-level lineage arrays; with ``max_ties`` the
    schedules of up to that many complete children tying for the best makespan."""
    mc = np.ascontiguousarray(machine, dtype=np.int32)
    du = np.ascontiguousarray(duration, dtype=np.int32)
    n, m = mc.shape
    N = n * m
    inst = _Instance(n, m, _ptr(mc), _ptr(du))
    tr = np.full((N, K), MARK, dtype=np.uint32) if trace else None
    tc = np.zeros(N, dtype=np.int32) if trace else None
    tbuf = np.zeros((max(max_ties, 0), N), dtype=np.int32)
    params = _Params(
        MODES[mode], K, best_known, seed & 0xFFFFFFFF,
        tr.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)) if trace else None,
        tc.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)) if trace else None,
        tbuf.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)) if max_ties > 0 else None,
        max(max_ties, 0),
    )
    seq = np.zeros(N, dtype=np.int32)
    res = _Result(0, 0, seq.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 0, 0, 0, 0)
    rc = _lib().orc_solve_levels(ctypes.byref(inst), ctypes.byref(params), ctypes.byref(res), max_levels)
    if rc != 0:
        raise ValueError(f"oracle rejected the input (status {rc})")
    out = dict(makespan=res.makespan, found=bool(res.found), seq=seq, expanded=res.expanded,
               slots=res.slots, levels=res.levels, ties=res.ties)
    if max_ties > 0:
        out["tie_seqs"] = tbuf[: min(res.ties, max_ties)]
    if trace:
        out["trace"] = tr
        out["trace_count"] = tc
    return out


def solve_iterations(machine, duration, mode: str, K: int, seeds, iterations: int,
                     initial_bound: int = 500000) -> dict:
    """Multi-start loop with the ranks as beams (orc_solve_iterations).  ``seeds`` is
    ``[iterations, beams]`` for the gpu modes and ``[beams]`` (srand seeds, the rand()
    stream carried across rounds) for ICH/PMS.  Returns best, seq and round_best."""
    mc = np.ascontiguousarray(machine, dtype=np.int32)
    du = np.ascontiguousarray(duration, dtype=np.int32)
    n, m = mc.shape
    sd = np.ascontiguousarray(np.asarray(seeds, dtype=np.int64) & 0xFFFFFFFF, dtype=np.uint32)
    beams = sd.shape[-1]
    inst = _Instance(n, m, _ptr(mc), _ptr(du))
    best = ctypes.c_int32()
    seq = np.zeros(n * m, dtype=np.int32)
    rounds = np.zeros(iterations, dtype=np.int32)
    rc = _lib().orc_solve_iterations(ctypes.byref(inst), MODES[mode], K, beams, iterations, _ptr(sd.ravel()),
                                     initial_bound, ctypes.byref(best), _ptr(seq), _ptr(rounds))
    if rc != 0:
        raise ValueError(f"oracle rejected the input (status {rc})")
    return dict(best=best.value, seq=seq, round_best=rounds)


def glibc_rand(seed: int, count: int) -> np.ndarray:
    out = np.zeros(count, dtype=np.int32)
    _lib().orc_glibc_rand_fill(seed & 0xFFFFFFFF, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), count)
    return out


def pivot_hash(x: int) -> int:
    return _lib().orc_pivot_hash(x & 0xFFFFFFFF)


def noise_hash(seed: int, c: int, b: int) -> int:
    return _lib().orc_noise_hash(seed & 0xFFFFFFFF, c & 0xFFFFFFFF, b & 0xFFFFFFFF)


def gpu_score(cmax: int, ns: int, seed: int, c: int, b: int) -> float:
    return _lib().orc_gpu_score(cmax, ns, seed & 0xFFFFFFFF, c & 0xFFFFFFFF, b & 0xFFFFFFFF)


def schedule_makespan(machine, duration, seq) -> int:
    mc = np.ascontiguousarray(machine, dtype=np.int32)
    du = np.ascontiguousarray(duration, dtype=np.int32)
    sq = np.ascontiguousarray(seq, dtype=np.int32)
    inst = _Instance(mc.shape[0], mc.shape[1], _ptr(mc), _ptr(du))
    return _lib().orc_schedule_makespan(ctypes.byref(inst), _ptr(sq))


# ---- the reference's own CPU solvers (present only where the reference tree is) ----
_ref = None


def ref_cpu_available() -> bool:
    return os.path.exists(REF_CPU_LIB)


def _reflib():
    global _ref
    if _ref is None:
        lib = ctypes.CDLL(REF_CPU_LIB)
        lib.ref_ich.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_uint]
        lib.ref_ich.restype = ctypes.c_int
        lib.ref_pms.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_uint]
        lib.ref_pms.restype = ctypes.c_int
        lib.ref_pms_iterations.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_uint, ctypes.c_int]
        lib.ref_pms_iterations.restype = ctypes.c_int
        P = ctypes.POINTER(ctypes.c_int)
        lib.ref_parse.argtypes = [ctypes.c_char_p, P, P, P, P, P, P, ctypes.c_int]
        lib.ref_parse.restype = ctypes.c_int
        lib.ref_resolve.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
        lib.ref_resolve.restype = ctypes.c_int
        _ref = lib
    return _ref


def ref_ich(path: str, K: int, seed: int) -> int:
    return _reflib().ref_ich(path.encode(), K, seed & 0xFFFFFFFF)


def ref_pms(path: str, K: int, best_known: int, seed: int) -> int:
    return _reflib().ref_pms(path.encode(), K, best_known, seed & 0xFFFFFFFF)


def ref_pms_iterations(path: str, K: int, seed: int, iterations: int) -> int:
    return _reflib().ref_pms_iterations(path.encode(), K, seed & 0xFFFFFFFF, iterations)


def ref_parse(path: str):
    cap = 1 << 16
    n, m, nbo = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    mc = (ctypes.c_int * cap)()
    du = (ctypes.c_int * cap)()
    jb = (ctypes.c_int * cap)()
    cnt = _reflib().ref_parse(path.encode(), ctypes.byref(n), ctypes.byref(m), ctypes.byref(nbo), mc, du, jb, cap)
    if cnt < 0:
        return None
    return dict(n=n.value, m=m.value, nboperation=nbo.value, machine1=list(mc[:cnt]),
                duration=list(du[:cnt]), job=list(jb[:cnt]))


def ref_resolve(arg: str):
    buf = ctypes.create_string_buffer(512)
    ok = _reflib().ref_resolve(arg.encode(), buf, 512)
    return buf.value.decode() if ok else None
