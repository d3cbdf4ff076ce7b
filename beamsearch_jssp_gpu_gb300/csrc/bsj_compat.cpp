// bsj_compat.cpp -- the reference-signature C++ entry points on top of the C ABI.
//
// run_gpu_beam_search_v1 / _v2 (gpu/v1/solver.cuh:6-12, gpu/v2_twophases/solver.cuh:6-12):
// converts the caller's JSSPInstance (1-based machines, dummy ops) to the C ABI's 0-based
// arrays, runs one beam on a per-device context kept for the life of the process, and
// maps errors to the reference's print-and-exit behaviour.
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/bsj.h"
#include "../../include/bsj_solver.h"

namespace {

std::mutex g_mu;        // the context table
std::mutex g_solve_mu;  // solves on the shared contexts
std::vector<bsj_context*> g_ctx;  // one per device, created on first use

bsj_context* device_context()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    std::lock_guard<std::mutex> lk(g_mu);
    if ((int)g_ctx.size() <= dev) g_ctx.resize(dev + 1, nullptr);
    if (!g_ctx[dev]) {
        bsj_context* c = nullptr;
        if (bsj_create(&c, dev) != BSJ_OK) {
            std::fprintf(stderr, "CUDA error %s:%d  cannot create a solver context on device %d\n",
                         __FILE__, __LINE__, dev);
            std::exit(EXIT_FAILURE);
        }
        g_ctx[dev] = c;
    }
    return g_ctx[dev];
}

int run_mode(int mode, const JSSPInstance& inst, int beam_width, int best_known, int random_seed,
             int* out_best_sequence)
{
    const int n = inst.nbjob, m = inst.nbmachine;
    if (n < 1 || m < 1 || (int)inst.operations.size() < n * m + 1) {
        std::fprintf(stderr, "Error: malformed JSSPInstance (n=%d m=%d, %zu operations)\n", n, m,
                     inst.operations.size());
        std::exit(EXIT_FAILURE);
    }
    std::vector<int32_t> mc((size_t)n * m), du((size_t)n * m);
    for (int q = 0; q < n * m; q++) {
        mc[q] = inst.operations[q + 1].num_mc - 1;
        du[q] = inst.operations[q + 1].dure;
    }
    bsj_instance bi{n, m, mc.data(), du.data()};
    bsj_beam bb{mode, beam_width, best_known, (uint32_t)random_seed, 0, -1};
    std::vector<int32_t> seq((size_t)n * m);
    bsj_result res{};
    res.sequence = seq.data();
    bsj_context* ctx = device_context();
    bsj_status s;
    {
        // one context per device is shared by every caller: calls are serialised (the
        // reference's entry points are not re-entrant either, gpu/common/gpu_common.cuh:32)
        std::lock_guard<std::mutex> lk(g_solve_mu);
        s = bsj_solve(ctx, &bi, &bb, &res, nullptr);
    }
    if (s != BSJ_OK) {
        std::fprintf(stderr, "CUDA error %s:%d  %s: %s\n", __FILE__, __LINE__, bsj_status_string(s),
                     bsj_last_error(ctx));
        std::exit(EXIT_FAILURE);
    }
    if (out_best_sequence != nullptr && res.makespan < BSJ_NO_BOUND) {
        for (int q = 0; q < n * m; q++) out_best_sequence[q] = seq[q];
    }
    return res.makespan;
}

}  // namespace

int run_gpu_beam_search_v1(const JSSPInstance& inst, int beam_width, int best_known,
                           int random_seed, int* out_best_sequence)
{
    return run_mode(BSJ_MODE_V1, inst, beam_width, best_known, random_seed, out_best_sequence);
}

int run_gpu_beam_search_v2(const JSSPInstance& inst, int beam_width, int best_known,
                           int random_seed, int* out_best_sequence)
{
    return run_mode(BSJ_MODE_V2, inst, beam_width, best_known, random_seed, out_best_sequence);
}
