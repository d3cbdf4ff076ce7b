"""ctypes binding of ``libbsj.so`` (include/bsj.h).

The library is the only compute path: if it is missing or cannot be loaded, every call
raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libbsj.so")

BSJ_OK = 0
BSJ_ERR_INVALID = 1
BSJ_ERR_LIMIT = 2
BSJ_ERR_CUDA = 3
BSJ_ERR_NOMEM = 4
BSJ_ERR_DEVICE = 5
STATUS_NAMES = {0: "ok", 1: "invalid argument", 2: "size outside the supported limits",
                3: "CUDA error", 4: "out of memory", 5: "device-side consistency check failed"}
MODES = {"v1": 0, "v2": 1, "clean": 2, "ich": 3, "pms": 4}
NO_BOUND = 500000
MAX_JOBS, MAX_MACHINES, MAX_OPS, MAX_BEAM = 128, 64, 8192, 16384

# Every symbol include/bsj.h declares (checked by the CPU tests without calling them).
EXPORTED = [
    "bsj_version", "bsj_status_string", "bsj_create", "bsj_destroy", "bsj_last_error",
    "bsj_solve", "bsj_solve_batch", "bsj_solve_iterations", "bsj_plan_create", "bsj_plan_run",
    "bsj_plan_results", "bsj_plan_destroy", "bsj_plan_launches", "bsj_plan_stats",
    "bsj_plan_set_timing", "bsj_plan_kernel_ms", "bsj_solve_noalloc",
    "bsj_instance_resolve", "bsj_instance_read", "bsj_schedule_decode", "bsj_device_count",
    "bsj_plan_estimate", "bsj_plan_device_bytes", "bsj_plan_update",
    "bsj_server_create", "bsj_server_destroy", "bsj_submit", "bsj_poll", "bsj_wait", "bsj_server_get_stats",
    "bsj_plan_autotune", "bsj_plan_set_chunk", "bsj_plan_chunk", "bsj_set_autotune",
    "bsj_plan_set_select_route", "bsj_plan_select_routes", "bsj_server_prepare", "bsj_plan_set_select_cluster",
]
# top-K selection routes (include/bsj.h BSJ_SELECT_* / BSJ_ROUTE_*)
SELECT = {"force_large": 1, "no_large": 2, "no_direct": 4, "radix": 8, "no_dense": 16, "rank_lsd": 32,
          "bitonic": 64, "no_cluster": 128, "force_cluster": 256}
ROUTE = {"large": 1, "direct": 2, "bucket": 4, "radix": 8, "dense": 16, "rank_lsd": 32, "raw_lsd": 64,
         "bitonic": 128, "cluster": 256}
CHUNK_SIZES = (8, 16, 32)  # k_step work-unit sizes (survivors per thread block), warp per survivor
GROUP_FORMS = (1, 2, 3, 4)  # k_step lane group per survivor: 4 lanes copy/bulk (1, 2), 8 lanes copy/bulk (3, 4)
CHUNK_CANDIDATES = (0, 8, 16, 32, 1, 2, 3, 4)  # the autotuner's candidates: 0 = the default rule


class ServerConfig(ctypes.Structure):
    _fields_ = [("max_inflight", ctypes.c_int32), ("cluster_inflight", ctypes.c_int32),
                ("memory_budget", ctypes.c_int64)]


class RequestTimes(ctypes.Structure):
    _fields_ = [("queue_ms", ctypes.c_double), ("run_ms", ctypes.c_double), ("built_plan", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class ServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in ("submitted", "completed", "plans_built", "plans_reused",
                                               "peak_inflight", "peak_device_bytes", "budget_bytes",
                                               "pending")] + \
               [(k, ctypes.c_double) for k in ("build_ms", "update_ms", "launch_ms", "collect_ms")] + \
               [("plans_prepared", ctypes.c_int64)]


class BsjError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Instance(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("m", ctypes.c_int32),
                ("machine", ctypes.POINTER(ctypes.c_int32)),
                ("duration", ctypes.POINTER(ctypes.c_int32))]


class Beam(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("beam_width", ctypes.c_int32),
                ("best_known", ctypes.c_int32), ("seed", ctypes.c_uint32),
                ("instance", ctypes.c_int32), ("bound_group", ctypes.c_int32)]


class Result(ctypes.Structure):
    _fields_ = [("makespan", ctypes.c_int32), ("found", ctypes.c_int32),
                ("sequence", ctypes.POINTER(ctypes.c_int32)),
                ("expanded", ctypes.c_int64), ("slots", ctypes.c_int64),
                ("levels", ctypes.c_int32), ("group_best", ctypes.c_int32)]


_lib: Optional[ctypes.CDLL] = None


def lib_path() -> str:
    return LIB_PATH


def load(path: Optional[str] = None) -> ctypes.CDLL:
    """Load libbsj.so (raising if it is absent: build it with
    ``python -c 'import __graft_entry__ as g; g.build()'``)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"libbsj.so not built ({p}); run beamsearch_jssp_gpu_gb300/build.py")
    L = ctypes.CDLL(p)
    vp = ctypes.c_void_p
    P = ctypes.POINTER
    L.bsj_version.restype = ctypes.c_char_p
    L.bsj_status_string.restype = ctypes.c_char_p
    L.bsj_status_string.argtypes = [ctypes.c_int]
    L.bsj_create.argtypes = [P(vp), ctypes.c_int]
    L.bsj_destroy.argtypes = [vp]
    L.bsj_destroy.restype = None
    L.bsj_last_error.argtypes = [vp]
    L.bsj_last_error.restype = ctypes.c_char_p
    L.bsj_solve.argtypes = [vp, P(Instance), P(Beam), P(Result), vp]
    L.bsj_solve_batch.argtypes = [vp, ctypes.c_int, P(Instance), ctypes.c_int, P(Beam), P(Result), vp]
    L.bsj_solve_iterations.argtypes = [vp, P(Instance), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, P(ctypes.c_uint32), ctypes.c_int32,
                                       P(ctypes.c_int32), P(ctypes.c_int32), P(ctypes.c_int32), vp]
    L.bsj_plan_create.argtypes = [vp, ctypes.c_int, P(Instance), ctypes.c_int, P(Beam), P(vp)]
    L.bsj_plan_run.argtypes = [vp, vp]
    L.bsj_plan_results.argtypes = [vp, P(Result)]
    L.bsj_plan_destroy.argtypes = [vp]
    L.bsj_plan_destroy.restype = None
    L.bsj_plan_launches.argtypes = [vp]
    L.bsj_plan_launches.restype = ctypes.c_int64
    L.bsj_plan_stats.argtypes = [vp, P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_int64),
                                 P(ctypes.c_int64), P(ctypes.c_int64)]
    L.bsj_plan_set_timing.argtypes = [vp, ctypes.c_int]
    L.bsj_plan_kernel_ms.argtypes = [vp, P(ctypes.c_float), P(ctypes.c_int64), ctypes.c_int]
    # autotuning of the k_step chunk size
    L.bsj_plan_autotune.argtypes = [vp, vp, ctypes.c_int32, P(ctypes.c_int32), P(ctypes.c_float)]
    L.bsj_plan_set_chunk.argtypes = [vp, ctypes.c_int32]
    L.bsj_plan_set_select_route.argtypes = [vp, ctypes.c_int32]
    L.bsj_plan_select_routes.argtypes = [vp, P(ctypes.c_uint32)]
    L.bsj_plan_chunk.argtypes = [vp]
    L.bsj_plan_chunk.restype = ctypes.c_int32
    L.bsj_set_autotune.argtypes = [vp, ctypes.c_int32]
    # allocation-free single-beam solve: device pointers in and out (include/bsj.h)
    L.bsj_solve_noalloc.argtypes = [ctypes.c_int32, ctypes.c_int32, vp, vp, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.c_int32, ctypes.c_uint32, vp, vp]
    L.bsj_solve_noalloc.restype = ctypes.c_int
    # host-side instance files and schedule decoding (no device needed)
    L.bsj_instance_resolve.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32]
    L.bsj_instance_read.argtypes = [ctypes.c_char_p, P(ctypes.c_int32), P(ctypes.c_int32),
                                    P(ctypes.c_int32), P(ctypes.c_int32), ctypes.c_int32]
    L.bsj_schedule_decode.argtypes = [P(Instance), P(ctypes.c_int32), P(ctypes.c_int32),
                                      P(ctypes.c_int32)]
    L.bsj_device_count.argtypes = [P(ctypes.c_int32)]
    L.bsj_plan_estimate.argtypes = [vp, ctypes.c_int, P(Instance), ctypes.c_int, P(Beam), P(ctypes.c_int64)]
    L.bsj_plan_device_bytes.argtypes = [vp]
    L.bsj_plan_device_bytes.restype = ctypes.c_int64
    L.bsj_plan_update.argtypes = [vp, ctypes.c_int, P(Instance), ctypes.c_int, P(Beam)]
    # serving (continuous batching)
    L.bsj_server_create.argtypes = [P(vp), ctypes.c_int, P(ServerConfig)]
    L.bsj_server_destroy.argtypes = [vp]
    L.bsj_server_destroy.restype = None
    L.bsj_submit.argtypes = [vp, P(Instance), P(Beam), P(ctypes.c_uint64)]
    L.bsj_poll.argtypes = [vp, ctypes.c_uint64, P(Result), P(RequestTimes), P(ctypes.c_int32)]
    L.bsj_wait.argtypes = [vp, ctypes.c_uint64, P(Result), P(RequestTimes)]
    L.bsj_server_get_stats.argtypes = [vp, P(ServerStats)]
    L.bsj_server_prepare.argtypes = [vp, P(Instance), P(Beam), ctypes.c_int32]
    for name in ("bsj_plan_estimate", "bsj_plan_update", "bsj_server_create", "bsj_submit", "bsj_poll",
                 "bsj_wait", "bsj_server_get_stats", "bsj_server_prepare"):
        getattr(L, name).restype = ctypes.c_int
    for name in ("bsj_instance_resolve", "bsj_instance_read", "bsj_schedule_decode", "bsj_device_count"):
        getattr(L, name).restype = ctypes.c_int
    for name in ("bsj_create", "bsj_solve", "bsj_solve_batch", "bsj_solve_iterations",
                 "bsj_plan_create", "bsj_plan_run", "bsj_plan_results", "bsj_plan_stats",
                 "bsj_plan_set_timing", "bsj_plan_kernel_ms", "bsj_plan_autotune", "bsj_plan_set_chunk",
                 "bsj_set_autotune", "bsj_plan_set_select_route", "bsj_plan_select_routes",
                 "bsj_plan_set_select_cluster"):
        getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L
