// bsj_device.cuh -- device-side layout, descriptors and per-state helpers shared by the
// level kernels.
//
// One beam entry ("snapshot") is a compact byte record, 16-byte aligned, that carries
// exactly what the reference's flat int snapshot (gpu/common/gpu_snapshot.cuh:8-31)
// needs for the next expansion:
//
//   off 0        int32 tr[m]      machine ready times (machine_ready_time, 0-based here)
//   off_jr       int32 jr[n]      finish time of each job's last scheduled op; this is
//                                 the only op_finish_time entry the reference ever reads
//                                 (op_finish_time[op-1], gpu_snapshot.cuh:58)
//   off_rd       u8    rd[n]      ready list as job ids, order significant
//                                 (precedence_ready_ops)
//   off_nx       u8    nx[n]      ops already scheduled per job (next op = j*m+nx[j]+1)
//   off_hdr      u16 r, u16 ns, int32 cmax, u32 lineage, u32 stamp
//
// The op sequence is not stored: every materialised entry appends (parent rank, job)
// to a per-level history, from which the best schedule is rebuilt once at the end.
// At 50x20 an entry is 400 B instead of the reference's 8 320 B.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace bsj {

enum Mode : int { MODE_V1 = 0, MODE_V2 = 1, MODE_CLEAN = 2, MODE_ICH = 3, MODE_PMS = 4 };

constexpr uint32_t kMark = 0xFFFFFFFFu;       // history value of a rank not rewritten
constexpr uint32_t kFillerFlag = 0x80000000u;  // selection entry that is a filler slot
constexpr int kMaxJobs = 128;
constexpr int kMaxMachines = 64;
constexpr int kMaxOps = 8192;
constexpr int kMaxBeam = 16384;
constexpr int kMaxDuration = (1 << 24) - 1;
constexpr int kSentinel = 500000;              // "no bound", gpu/v1/main.cu:57
constexpr int kWarpsPerStepCta = 8;
// k_step work unit: a chunk of consecutive ranks of one beam per CTA, 1, 2 or 4 ranks per
// warp.  The chunk size is chosen per plan (StepArgs::chunk) among kChunkSizes, by the
// autotuner or by the default rule; candidate keys and per-chunk counts are laid out for
// every size (keys for the largest, counts for the smallest).
constexpr int kNumChunkSizes = 3;
constexpr int kChunkSizes[kNumChunkSizes] = {8, 16, 32};
constexpr int kMinChunk = 8;
constexpr int kMaxChunk = 32;
constexpr int kDefaultChunk = 16;   // ranks per k_step CTA when nothing else decides
constexpr int kMaxChunks = kMaxBeam / kMinChunk;
static_assert(kMinChunk % kWarpsPerStepCta == 0 && kMaxChunk <= 32, "a chunk is 1..4 ranks per warp");
constexpr int kSelectThreads = 1024;
constexpr int kHeapThreads = 256;    // k_heap: warp 0 runs the heap, warps 1..7 prepare chunks
constexpr int kHeapMaxChunk = 32;     // parents per k_heap chunk (at most)

// Device-side error bits (SegState::status).
constexpr int kStatusBadLineage = 1;
constexpr int kStatusBadSelect = 2;

// Routes of k_select's top-K selection.  StepArgs::select_force (0 = the normal choice by
// level size) forces a level onto a route, so tests can run every route on small
// levels; the result never depends on the route.
constexpr int kSelForceLarge = 1;   // global-memory large-level path whatever the level size
constexpr int kSelNoLarge = 2;      // never the large-level path
constexpr int kSelNoDirect = 4;     // no direct staged path: compact the survivors first
constexpr int kSelForceRadix = 8;   // MSD radix select of the R-th key, not the bucket threshold
constexpr int kSelNoDense = 16;     // LSD passes on the raw score bits (no dense ranks)
constexpr int kSelRankLsd = 32;     // dense ranks written into the keys, then LSD passes
constexpr int kSelBitonic = 64;     // block bitonic sort of the survivors
constexpr int kSelNoCluster = 128;  // one CTA per beam (no cluster select launch)
constexpr int kSelForceCluster = 256;  // cluster launch, and its route on every level it can take
constexpr int kSelAll = 511;
// Routes the levels of a beam took (SegState::select_paths, OR over the levels).
constexpr uint32_t kPathLarge = 1, kPathDirect = 2, kPathBucket = 4, kPathRadix = 8, kPathDense = 16,
                   kPathRankLsd = 32, kPathRawLsd = 64, kPathBitonic = 128, kPathCluster = 256;
// The cluster select: launched for beams of K >= kSelectClusterMinK, its route taken on
// levels of more than kClusterMinKeys keys, 2 CTAs per beam, or 4 where K * n reaches
// kSelectClusterWideKN (levels of ~15 K keys and more).  Measured on GB300 (ms per search):
// one block / 2 CTAs: 50x20 K=4096 28.3 / 25.5, 20x15 K=4096 7.37 / 6.97, 100x20 K=4096
// 100.1 / 69.5 (taking only levels above 8 192 keys was slower on every shape; launching
// it for K=2048 at 20x15, levels of ~4.5 K keys, slower than one block); 2 / 4 CTAs:
// 50x20 K=4096 24.98 / 24.06 (8 beams 27.81 / 27.73), 100x20 K=4096 66.52 / 63.21, 30x20
// K=4096 13.95 / 14.00, 20x15 K=4096 6.86 / 7.01.
constexpr int kSelectClusterMinK = 4096;
constexpr int kClusterMinKeys = 4096;
constexpr int kSelectClusterWideKN = 150000;

struct SegDesc {
    int32_t n, m, N, K;
    int32_t mode;
    uint32_t seed;
    int32_t sbytes, off_jr, off_rd, off_nx, off_hdr;
    int32_t words;      // mask words per parent (ceil(n/32))
    int32_t group;      // bound group
    int32_t auxbytes;   // per-parent bytes of the ICH/PMS child table
    int32_t op_off;     // index of this instance in the op table
    int32_t nq;         // ceil(n / 32): 32-lane groups a warp needs for the ready list
    int32_t kcnt_off;   // index of this beam's first per-chunk key count
    int32_t pad1;
    int64_t beam_off[2];  // byte offsets of the two beam buffers
    int64_t slot_off;     // byte offset of the v1 child-slot buffer
    int64_t key_off;      // u64 index: candidate keys of the current level
    int64_t sel_off;      // u32 index: selected survivors
    int64_t mask_off;     // u32 index: per-parent scored-branch masks
    int64_t hist_off;     // u32 index: per-level (parent << 8 | job) history
    int64_t aux_off;      // byte offset: ICH/PMS per-parent child table
    int64_t seq_off;      // i32 index: result sequence
    int64_t pos_off[2];   // byte offsets (gpu-v2/clean): per state and branch b, the ready-list
                          // position of branch b's op (0xFF past the last branch); ping-pong by
                          // level parity
};

struct SegState {
    int32_t P;            // beam entries at the current level
    int32_t V;            // candidate keys written for the current level
    int32_t bound;        // frozen pruning bound (best_known of this pass)
    int32_t status;
    unsigned long long best;  // gpu modes: (cmax << 32) | (slot << 8) | job
    uint32_t best_ref;        // ICH/PMS: (parent << 8) | job of the best complete child
    int32_t best_cmax;        // ICH/PMS: its makespan (kSentinel if none)
    long long expanded;
    long long slots;
    long long materialized;   // survivors materialised (sum of beam sizes after each level)
    long long select_fallbacks;  // levels whose top-K took the radix-select path
    int32_t levels;
    int32_t makespan;
    int32_t found;
    uint32_t select_paths;  // kPath* bits of the selection routes taken
    uint32_t rng_i;       // ICH/PMS rand() stream: position of the next value, in [34, 68)
    uint32_t rng[34];
};

// ---- hashes of the gpu solvers (gpu/v1/solver.cu:51-54, :121-126) ----
__device__ __forceinline__ uint32_t pivot_hash(uint32_t h)
{
    h ^= h >> 16; h *= 0x7feb352du;
    h ^= h >> 15; h *= 0x846ca68bu;
    h ^= h >> 16;
    return h;
}

__device__ __forceinline__ uint32_t noise_hash(uint32_t seed, uint32_t c, uint32_t b)
{
    uint32_t h = seed ^ (c * 0x85ebca6bu) ^ (b * 0xc2b2ae35u);
    h ^= h >> 16; h *= 0x85ebca6bu;
    h ^= h >> 16; h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

// fp32 score of the gpu solvers, IEEE round-to-nearest division as built without
// fast-math (gpu/v1/solver.cu:121-127; reference Makefile:40).
__device__ __forceinline__ float gpu_score(int cmax, int ns, uint32_t seed, uint32_t c, uint32_t b)
{
    float base = __fdiv_rn(__int2float_rn(cmax), __int2float_rn(ns));
    float noise = __fdiv_rn(__uint2float_rn(noise_hash(seed, c, b) % 1000u), 1000000000.0f);
    return __fadd_rn(base, noise);
}

// ---- snapshot field access on a (shared-memory) byte buffer ----
struct Lay {
    int n, m, off_jr, off_rd, off_nx, off_hdr, sbytes;
    __device__ __forceinline__ explicit Lay(const SegDesc& d)
        : n(d.n), m(d.m), off_jr(d.off_jr), off_rd(d.off_rd), off_nx(d.off_nx),
          off_hdr(d.off_hdr), sbytes(d.sbytes) {}
};

__device__ __forceinline__ int32_t* TR(uint8_t* b) { return reinterpret_cast<int32_t*>(b); }
__device__ __forceinline__ int32_t* JR(uint8_t* b, const Lay& L) { return reinterpret_cast<int32_t*>(b + L.off_jr); }
__device__ __forceinline__ uint8_t* RD(uint8_t* b, const Lay& L) { return b + L.off_rd; }
__device__ __forceinline__ uint8_t* NX(uint8_t* b, const Lay& L) { return b + L.off_nx; }
__device__ __forceinline__ uint16_t* H_R(uint8_t* b, const Lay& L) { return reinterpret_cast<uint16_t*>(b + L.off_hdr); }
__device__ __forceinline__ uint16_t* H_NS(uint8_t* b, const Lay& L) { return reinterpret_cast<uint16_t*>(b + L.off_hdr + 2); }
__device__ __forceinline__ int32_t* H_CMAX(uint8_t* b, const Lay& L) { return reinterpret_cast<int32_t*>(b + L.off_hdr + 4); }
__device__ __forceinline__ uint32_t* H_LIN(uint8_t* b, const Lay& L) { return reinterpret_cast<uint32_t*>(b + L.off_hdr + 8); }
__device__ __forceinline__ uint32_t* H_STAMP(uint8_t* b, const Lay& L) { return reinterpret_cast<uint32_t*>(b + L.off_hdr + 12); }

// Warp-cooperative 16-byte copies (sbytes is a multiple of 16, buffers 16-byte aligned).
__device__ __forceinline__ void warp_load(uint8_t* dst_smem, const uint8_t* src_gmem, int sbytes, int lane)
{
    const uint4* s = reinterpret_cast<const uint4*>(src_gmem);
    uint4* d = reinterpret_cast<uint4*>(dst_smem);
    for (int q = lane; q < (sbytes >> 4); q += 32) d[q] = __ldg(s + q);
}

__device__ __forceinline__ void warp_store(uint8_t* dst_gmem, const uint8_t* src_smem, int sbytes, int lane)
{
    const uint4* s = reinterpret_cast<const uint4*>(src_smem);
    uint4* d = reinterpret_cast<uint4*>(dst_gmem);
    for (int q = lane; q < (sbytes >> 4); q += 32) d[q] = s[q];
}

__device__ __forceinline__ void warp_copy_smem(uint8_t* dst, const uint8_t* src, int sbytes, int lane)
{
    const uint4* s = reinterpret_cast<const uint4*>(src);
    uint4* d = reinterpret_cast<uint4*>(dst);
    for (int q = lane; q < (sbytes >> 4); q += 32) d[q] = s[q];
}

}  // namespace bsj
