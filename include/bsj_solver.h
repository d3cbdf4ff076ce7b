// bsj_solver.h -- C++ drop-in for the reference's GPU solver entry points.
//
// Same names, signatures, argument meaning, return value and error behaviour as
//   gpu/v1/solver.cuh:6-12          int run_gpu_beam_search_v1(...)
//   gpu/v2_twophases/solver.cuh:6-12 int run_gpu_beam_search_v2(...)
// so that the reference's drivers (gpu/v1/main.cu:64, gpu/v1/benchmark.cu:61,
// hybrid/v1/solver.cu:29 and their v2 twins) link against libbsj.so unchanged.
//
// The instance types restate cpu/common/jssp_types.h:8-23 member for member (the types
// are part of the mangled signature and of the object layout the callers pass in).  A
// translation unit includes either this header or the reference's jssp_types.h, never
// both.
#pragma once

#include <vector>

struct Operation {
    int num_op;  // 1-indexed operation id
    int num_mc;  // 1-indexed machine id
    int dure;    // processing duration
    int num_j;   // 1-indexed job id
};

struct JSSPInstance {
    int nbjob = 0;
    int nbmachine = 0;
    int nboperation = 0;
    std::vector<Operation> operations;        // [nboperation], dummies at 0 and n*m+1
    std::vector<std::vector<int>> opr_mach;   // unused by the solvers
};

// One GPU beam-search pass, gpu/v1 semantics bit for bit.  Returns
// min(best_known, best complete makespan); writes the best schedule's 1-based op ids
// into out_best_sequence[0 .. n*m) when it is non-null and the result is < 500000.
// On a CUDA or input error prints a message and exits with EXIT_FAILURE, as the
// reference's CUDA_CHECK does (gpu/common/gpu_common.cuh:9-17); use the C ABI (bsj.h)
// for status codes instead.
int run_gpu_beam_search_v1(const JSSPInstance& inst, int beam_width, int best_known,
                           int random_seed, int* out_best_sequence = nullptr);

// Same contract with gpu/v2_twophases semantics.
int run_gpu_beam_search_v2(const JSSPInstance& inst, int beam_width, int best_known,
                           int random_seed, int* out_best_sequence = nullptr);

// The instance reader of cpu/common/instance_parser.h:5-9, same signatures and behaviour
// (instance_parser.cpp:8-34, :37-93): resolve_instance_file tries the argument as a path,
// then the reference's list of Lawrence/Taillard locations; parse_instance fills `inst`
// with dummy ops 0 and n*m+1 and 1-based machines, and prints to stderr and returns
// false when the file cannot be opened or its header read.
bool resolve_instance_file(const char* input_arg, char* out_path, int path_size);
bool parse_instance(const char* filepath, JSSPInstance& inst);
