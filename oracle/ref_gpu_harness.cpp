// ref_gpu_harness.cpp -- TEST INFRASTRUCTURE: runs the reference's own gpu kernels.
//
// The reference's device code (gpu/v1/solver.cu, gpu/v2_twophases/solver.cu) is compiled
// from its sources into oracle/_ref/ref_gpu_v{1,2}.cubin by oracle/Makefile.  This
// program loads that cubin with the CUDA driver API and drives the kernels with a
// restatement of the reference host loop (run_gpu_beam_search_v1, gpu/v1/solver.cu:178-298;
// run_gpu_beam_search_v2, gpu/v2_twophases/solver.cu:256-386).  The one substitution is
// the sort: the reference's cub::DeviceRadixSort::SortPairs (stable, ascending float keys)
// becomes a host std::stable_sort of the same (score, slot) pairs, which has the same
// unique result.  All device buffers are zeroed first, as a fresh process's first
// allocation reads.
//
// Usage: ref_gpu_harness v1|v2 <cubin> <instance file> <K> <best_known> <seed> [time]
// Prints one JSON object: {"makespan": M, "sequence": [...]}; with `time`, also the device
// time of the reference's two kernels summed over the search (CUDA events around every
// launch), "kernel_ms": [first, second], and the host time of the substituted sort,
// "host_sort_ms" -- a lower bound of the reference's own GPU time, which adds CUB's sort.
#include <cuda.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#define CK(call)                                                                  \
    do {                                                                          \
        CUresult _r = (call);                                                     \
        if (_r != CUDA_SUCCESS) {                                                 \
            const char* _s = nullptr;                                             \
            cuGetErrorString(_r, &_s);                                            \
            std::fprintf(stderr, "driver error %d (%s) at %s:%d\n", (int)_r,      \
                         _s ? _s : "?", __FILE__, __LINE__);                      \
            std::exit(2);                                                         \
        }                                                                         \
    } while (0)

// gpu/common/gpu_snapshot.cuh:8-31 (passed by value to the kernels).
struct Layout {
    int off_machine_ready, off_op_finish, off_precedence_ready, off_ready_count;
    int off_sequence, off_sequence_count, off_makespan, total_ints;
};

static Layout make_layout(int num_jobs, int num_machines, int num_ops)
{
    Layout L;
    L.off_machine_ready = 0;
    L.off_op_finish = L.off_machine_ready + (num_machines + 1);
    L.off_precedence_ready = L.off_op_finish + (num_ops + 1);
    L.off_ready_count = L.off_precedence_ready + num_jobs;
    L.off_sequence = L.off_ready_count + 1;
    L.off_sequence_count = L.off_sequence + (num_ops + 1);
    L.off_makespan = L.off_sequence_count + 1;
    L.total_ints = L.off_makespan + 1;
    return L;
}

struct OpInfo { int machine_id, duration, job_id; };  // gpu_common.cuh:25-29

static CUfunction find_kernel(CUmodule mod, const char* needle)
{
    unsigned cnt = 0;
    CK(cuModuleGetFunctionCount(&cnt, mod));
    std::vector<CUfunction> fs(cnt);
    CK(cuModuleEnumerateFunctions(fs.data(), cnt, mod));
    for (CUfunction f : fs) {
        const char* nm = nullptr;
        CK(cuFuncGetName(&nm, f));
        if (nm && std::strstr(nm, needle)) return f;
    }
    std::fprintf(stderr, "kernel %s not found in module\n", needle);
    std::exit(2);
}

int main(int argc, char** argv)
{
    if (argc != 7 && !(argc == 8 && std::string(argv[7]) == "time")) {
        std::fprintf(stderr, "usage: %s v1|v2 cubin instance K best_known seed [time]\n", argv[0]);
        return 1;
    }
    const bool timing = argc == 8;
    const bool v2 = std::string(argv[1]) == "v2";
    const int K = std::atoi(argv[4]);
    const int best_known = std::atoi(argv[5]);
    const int seed = (int)std::strtoll(argv[6], nullptr, 10);

    // instance text format (cpu/common/instance_parser.cpp:37-93)
    FILE* f = std::fopen(argv[3], "r");
    if (!f) { std::fprintf(stderr, "cannot open %s\n", argv[3]); return 1; }
    int n = 0, m = 0;
    if (std::fscanf(f, "%d %d", &n, &m) != 2) return 1;
    const int nbop = n * m + 2, N = n * m;
    std::vector<OpInfo> ops(nbop, OpInfo{0, 0, 0});
    for (int j = 0; j < n; j++)
        for (int k = 0; k < m; k++) {
            int mc = 0, du = 0;
            if (std::fscanf(f, "%d %d", &mc, &du) != 2) { mc = 0; du = 0; }
            ops[j * m + k + 1] = OpInfo{mc + 1, du, j + 1};
        }
    std::fclose(f);

    CK(cuInit(0));
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    CUmodule mod;
    CK(cuModuleLoad(&mod, argv[2]));
    CUfunction k_first = find_kernel(mod, v2 ? "kernel_score_candidates" : "kernel_expand_beam_layer");
    CUfunction k_second = find_kernel(mod, v2 ? "kernel_materialize_topk" : "kernel_gather_topk");

    // copy_instance_to_device (gpu_common.cuh:35-46)
    CUdeviceptr c_ops;
    size_t c_ops_bytes = 0;
    CK(cuModuleGetGlobal(&c_ops, &c_ops_bytes, mod, "c_ops"));
    const size_t cnt_ops = std::min<size_t>((size_t)nbop, c_ops_bytes / sizeof(OpInfo));
    CK(cuMemcpyHtoD(c_ops, ops.data(), cnt_ops * sizeof(OpInfo)));

    const Layout L = make_layout(n, m, nbop);
    const size_t S = (size_t)L.total_ints;
    const size_t max_children = (size_t)K * n;
    CUdeviceptr beam_a, beam_b = 0, child = 0, scores, indices, sorted, gbest, best_sol;
    CK(cuMemAlloc(&beam_a, (size_t)K * S * 4));
    if (v2) CK(cuMemAlloc(&beam_b, (size_t)K * S * 4));
    else CK(cuMemAlloc(&child, max_children * S * 4));
    CK(cuMemAlloc(&scores, max_children * 4));
    CK(cuMemAlloc(&indices, max_children * 4));
    CK(cuMemAlloc(&sorted, max_children * 4));
    CK(cuMemAlloc(&gbest, 4));
    CK(cuMemAlloc(&best_sol, S * 4));
    CK(cuMemsetD8(beam_a, 0, (size_t)K * S * 4));
    if (v2) CK(cuMemsetD8(beam_b, 0, (size_t)K * S * 4));
    else CK(cuMemsetD8(child, 0, max_children * S * 4));
    CK(cuMemsetD8(scores, 0, max_children * 4));
    CK(cuMemsetD8(indices, 0, max_children * 4));
    CK(cuMemsetD8(best_sol, 0, S * 4));
    CK(cuMemcpyHtoD(gbest, &best_known, 4));

    // pack_initial_snapshot (gpu_snapshot.cuh:34-44)
    std::vector<int> root(S, 0);
    for (int j = 0; j < n; j++) root[L.off_precedence_ready + j] = j * m + 1;
    root[L.off_ready_count] = n;
    CK(cuMemcpyHtoD(beam_a, root.data(), S * 4));

    CUevent ev[4];
    for (CUevent& e : ev) CK(cuEventCreate(&e, CU_EVENT_DEFAULT));
    double kms[2] = {0.0, 0.0}, sort_ms = 0.0;
    auto elapsed = [&](CUevent a, CUevent b) {
        float t = 0.f;
        CK(cuEventElapsedTime(&t, a, b));
        return (double)t;
    };
    CUdeviceptr cur = beam_a, nxt = beam_b;
    int P = 1;
    const unsigned smem = (unsigned)((S + n + 1) * 4);
    std::vector<float> h_scores(max_children);
    std::vector<int> h_idx(max_children), h_sorted(max_children), order(max_children);
    for (int step = 0; step < N; step++) {
        const int total = P * n;
        int step_seed = (int)((unsigned)seed + (unsigned)step);
        int num_machines = m, num_ops_tot = nbop, total_real = N, bpc = n;
        Layout lay = L;
        if (timing) CK(cuEventRecord(ev[0], 0));
        if (!v2) {
            void* args[] = {&cur, &child, &scores, &indices, &gbest, &best_sol, &P, &bpc, &lay,
                            &num_machines, &num_ops_tot, &total_real, &step_seed};
            CK(cuLaunchKernel(k_first, P, 1, 1, n, 1, 1, smem, 0, args, nullptr));
        } else {
            void* args[] = {&cur, &scores, &indices, &gbest, &best_sol, &P, &bpc, &lay,
                            &num_machines, &num_ops_tot, &total_real, &step_seed};
            CK(cuLaunchKernel(k_first, P, 1, 1, n, 1, 1, smem, 0, args, nullptr));
        }
        if (timing) CK(cuEventRecord(ev[1], 0));
        CK(cuCtxSynchronize());
        if (timing) kms[0] += elapsed(ev[0], ev[1]);
        const auto t_sort = std::chrono::steady_clock::now();
        CK(cuMemcpyDtoH(h_scores.data(), scores, (size_t)total * 4));
        CK(cuMemcpyDtoH(h_idx.data(), indices, (size_t)total * 4));
        std::iota(order.begin(), order.begin() + total, 0);
        std::stable_sort(order.begin(), order.begin() + total,
                         [&](int x, int y) { return h_scores[x] < h_scores[y]; });
        for (int r = 0; r < total; r++) h_sorted[r] = h_idx[order[r]];
        CK(cuMemcpyHtoD(sorted, h_sorted.data(), (size_t)total * 4));
        sort_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_sort).count();
        int gather = std::min(total, K);
        if (timing) CK(cuEventRecord(ev[2], 0));
        int threads = 256, blocks = (gather + threads - 1) / threads;
        if (!v2) {
            int sints = (int)S;
            void* args[] = {&child, &sorted, &cur, &gather, &sints};
            CK(cuLaunchKernel(k_second, blocks, 1, 1, threads, 1, 1, 0, 0, args, nullptr));
        } else {
            void* args[] = {&cur, &sorted, &nxt, &gather, &bpc, &lay, &num_machines, &num_ops_tot,
                            &step_seed};
            CK(cuLaunchKernel(k_second, blocks, 1, 1, threads, 1, 1, 0, 0, args, nullptr));
            std::swap(cur, nxt);
        }
        if (timing) CK(cuEventRecord(ev[3], 0));
        CK(cuCtxSynchronize());
        if (timing) kms[1] += elapsed(ev[2], ev[3]);
        P = gather;
    }
    int best = 500000;
    CK(cuMemcpyDtoH(&best, gbest, 4));
    std::vector<int> sol(S, 0);
    CK(cuMemcpyDtoH(sol.data(), best_sol, S * 4));
    std::printf("{\"makespan\": %d, \"sequence\": [", best);
    for (int t = 0; t < N; t++) std::printf("%s%d", t ? ", " : "", best < 500000 ? sol[L.off_sequence + t] : 0);
    if (timing) std::printf("], \"kernel_ms\": [%.3f, %.3f], \"host_sort_ms\": %.3f}\n", kms[0], kms[1], sort_ms);
    else std::printf("]}\n");
    for (CUevent& e : ev) CK(cuEventDestroy(e));
    CK(cuModuleUnload(mod));
    CK(cuDevicePrimaryCtxRelease(dev));
    return 0;
}
