"""GB300-native beam search for the job-shop scheduling problem.

A drop-in for the solver interface of bensdz/BeamSearch_JSSP_GPU: the same instance text
format, the ``run_gpu_beam_search_v1/v2`` entry points (C ABI in include/bsj.h, C++
signatures in include/bsj_solver.h, Python mirror in :mod:`.solver`), beam width K,
branching mode and seed.  One search level runs as hand-written sm_103a CUDA kernels in
``_lib/libbsj.so``; there is no CPU compute path.
"""
from .instance import (JSSPInstance, Operation, format_instance, parse_instance,  # noqa: F401
                       resolve_instance_file, schedule_makespan, synthetic_instance,
                       write_instance)
from .solver import (BeamSpec, Context, Plan, Server, beam_search_ich, beam_search_pms,  # noqa: F401
                     run_gpu_beam_search_v1, run_gpu_beam_search_v2, solve, solve_batch,
                     solve_iterations)
from ._native import BsjError, NO_BOUND, MODES  # noqa: F401

__version__ = "0.1.0"
