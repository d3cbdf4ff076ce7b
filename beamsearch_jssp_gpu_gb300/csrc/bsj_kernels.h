// bsj_kernels.h -- launch interface between the host engine and the level kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "bsj_device.cuh"

namespace bsj {

// Everything a level kernel needs, passed by value (fits the kernel parameter space).
struct StepArgs {
    const SegDesc* segs;
    SegState* st;
    const int32_t* rank_prefix;   // [nseg+1] prefix sums of K (flattened rank space)
    const int32_t* chunk_prefix;  // [nseg+1] prefix sums of ceil(K/chunk)
    int32_t* kcnt;                // candidate keys per chunk of the current level
    uint2* kmm;                   // per chunk of the current level: min / max score bits of
                                  // its keys ({~0, 0} when it has none)
    int32_t nseg;
    int32_t total_ranks;
    int32_t total_chunks;
    int32_t sb_max;               // per-warp state buffer bytes (max sbytes)
    int32_t max_n;                // largest n of the batch (k_step key staging)
    // the beams this launch works on: [seg_lo, seg_hi) and their chunk / rank ranges
    // (several ranges run as independent branches of one graph)
    int32_t seg_lo, seg_hi;
    int32_t chunk_lo, chunk_hi;
    int32_t rank_lo, rank_hi;
    int32_t chunk;                // ranks per k_step CTA (one of kChunkSizes)
    int32_t select_force;         // kSel* route flags for k_select (0 = by level size)
    int32_t group_step;           // k_step form: 0 warp per survivor; 1-4 a lane group per
                                  // survivor (k_step_g: 4 lanes copy / bulk, 8 lanes copy / bulk)
    int32_t select_cluster;       // CTAs per beam of k_select: 1, or 2 / 4 (cluster launch)
    uint8_t* beam_pool;
    uint8_t* slot_pool;
    unsigned long long* keys;
    uint32_t* sel;
    uint32_t* masks;
    uint32_t* hist;
    uint8_t* aux_pool;
    const uint32_t* ops;          // (duration << 8) | machine per op, per instance
    int32_t* group_best;
    int32_t* seq_pool;
    uint8_t* pos_pool;            // branch -> ready position tables (SegDesc::pos_off)
    const float* noise;           // [1000]: (float)k / 1e9f, IEEE round-to-nearest
    const double* dnoise;         // [1000]: (double)k / 1e6 (BS-PMS noise), IEEE round-to-nearest
};

// k_step variants (the autotuner's candidates besides the default rule): a warp per
// survivor with 8, 16 or 32 survivors per CTA; a group of 4 lanes per survivor (32 per
// CTA) or of 8 lanes (16 per CTA), the parent snapshots staged by the group's 16-byte
// copies or by one bulk copy.  Group variants apply to beam groups whose beams are all
// gpu-v2 / clean; other groups run the warp kernel with the same chunk size.  Public
// codes (bsj_plan_set_chunk): 8, 16, 32 (warp), 1, 2, 3, 4 (group).
constexpr int kNumStepVariants = 7;
constexpr int kStepVariantChunk[kNumStepVariants] = {8, 16, 32, 32, 32, 16, 16};
constexpr int kStepVariantGroup[kNumStepVariants] = {0, 0, 0, 1, 2, 3, 4};
constexpr int kStepVariantCode[kNumStepVariants] = {8, 16, 32, 1, 2, 3, 4};

// k_heap launch configuration: the largest K, child-table row (bytes) and n of the
// launch's ICH/PMS beams, and the parents prepared per chunk.
struct HeapCfg {
    int32_t kmax, chunk, ab, nmax;
};

// Grid / shared-memory sizing helpers.
size_t step_smem_bytes(int sb_max, int max_n, int chunk);
size_t select_smem_bytes(int sort_cap);
size_t heap_smem_bytes(const HeapCfg& c);
// Largest chunk in [1, kHeapMaxChunk] whose k_heap shared memory fits `budget`; 0 if none.
int heap_pick_chunk(HeapCfg c, size_t budget);

// Launchers (asynchronous on `stream`).
// k_step is instantiated per NQ = ceil(n/32) in {1, 2, 4} and chunk size (a.chunk);
// nq_mask has bit NQ set for each class present in the batch (one launch per class).
cudaError_t launch_step(const StepArgs& a, int s, int grid, int nq_mask, cudaStream_t stream);
int nq_class(int n);
cudaError_t launch_gather_v1(const StepArgs& a, int s, int grid, cudaStream_t stream);
cudaError_t launch_select(const StepArgs& a, int s, int sort_cap, cudaStream_t stream);
cudaError_t launch_heap(const StepArgs& a, int s, const HeapCfg& hc, cudaStream_t stream);
// Fills noise[0..1000) with (float)k / 1e9f (once per plan; k_step copies it per CTA).
cudaError_t launch_noise_table(float* noise, double* dnoise, cudaStream_t stream);
cudaError_t launch_finalize(const StepArgs& a, cudaStream_t stream);
cudaError_t configure_kernels(int sort_cap, const HeapCfg* hc, int sb_max, int max_n);
// Raise (never lower) the dynamic shared-memory limits of k_select and k_step to what
// a launch with `sort_cap` / `sb_max` needs.
cudaError_t raise_kernel_smem(int sort_cap, int sb_max, int max_n);

}  // namespace bsj
