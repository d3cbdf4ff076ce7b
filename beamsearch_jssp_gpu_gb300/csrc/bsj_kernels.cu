// bsj_kernels.cu -- the level kernels of the beam search, sm_103a.
//
// One search level (reference: the body of the level loop, gpu/v1/solver.cu:234-275 and
// gpu/v2_twophases/solver.cu:315-363) runs as
//
//   k_select(s)      per beam: exact top-K of the level's candidate keys + stable order
//                    (replaces cub::DeviceRadixSort::SortPairs over all P*n slots)
//   k_heap(s)        per beam, ICH/PMS modes: the CPU solvers' bounded heap, in order
//   k_gather_v1(s)   v1 mode only: copy the selected child slots into the beam
//   k_step(s)        warp per survivor: materialise the survivor from its parent (fused
//                    gather), then expand it for level s+1: pivot machine by ballot,
//                    child makespan, fp32 score, key emission
//
// Integer work only, apart from the fp32 (gpu modes) / fp64 (PMS) score, computed with
// the reference's operations in its order.
#include <mutex>

#include "bsj_kernels.h"

namespace bsj {

#define FULL_MASK 0xFFFFFFFFu

// ------------------------------------------------------------------------------------
// helpers
// ------------------------------------------------------------------------------------
// The beam holding flat index `flat` among the launch's beams [lo, hi) (prefix = per-beam
// prefix sums).  A launch is usually one beam group of few beams -- often one -- so the
// search is over that range, not over every beam of the plan.
__device__ __forceinline__ int find_seg(const int32_t* prefix, int lo, int hi, int flat)
{
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (__ldg(prefix + mid) <= flat) lo = mid; else hi = mid;
    }
    return lo;
}

// The beam descriptor (constant for a plan, written before its first launch) pulled into L1
// before the selection waits on its producer, so its reads after the wait hit.  (In k_step,
// whose CTAs are many and short, the same prefetch measured slower.)
__device__ __forceinline__ void prefetch_desc(const SegDesc* d)
{
    const char* p = reinterpret_cast<const char*>(d);
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p + 128));
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p + sizeof(SegDesc) - 1));
}
static_assert(sizeof(SegDesc) > 128, "prefetch_desc touches offsets 0, 128 and the last byte");

__device__ __forceinline__ uint32_t op_info(const uint32_t* ops, int op_off, int j, int m, int k)
{
    return __ldg(ops + op_off + j * m + k);
}

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// A warp's min / max score bits into the chunk's range (s_mm[0] min, s_mm[1] max): the
// selection takes the level's score range from these instead of a pass over its keys.
__device__ __forceinline__ void chunk_range_add(uint32_t mn, uint32_t mx, uint32_t* s_mm, int lane)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = min(mn, __shfl_xor_sync(FULL_MASK, mn, o));
        mx = max(mx, __shfl_xor_sync(FULL_MASK, mx, o));
    }
    if (lane == 0 && mn <= mx) {
        atomicMin(&s_mm[0], mn);
        atomicMax(&s_mm[1], mx);
    }
}

// Programmatic dependent launch.  The level kernels are launched with programmatic stream
// serialization and wait (griddepcontrol.wait) for their predecessor's completion and
// memory before touching anything it wrote.  k_step also lets its successor -- the next
// level's select or heap -- be scheduled as soon as it starts, so those few CTAs are
// resident when k_step ends.  The narrow kernels trigger late or not at all: the wide
// k_step grid after them would otherwise sit on SM slots other beams need (the cluster
// select triggers before its last phase).  Without the launch attribute both instructions
// are no-ops.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Warp-wide asynchronous copy of one snapshot into shared memory (16-byte pieces).
__device__ __forceinline__ void warp_prefetch(uint8_t* dst_smem, const uint8_t* src_gmem, int sbytes, int lane)
{
    for (int q = lane; q < (sbytes >> 4); q += 32) cp_async16(dst_smem + 16 * q, src_gmem + 16 * q);
}

// Root state: first op of every job ready in job order (gpu_snapshot.cuh:34-44,
// jssp_types.h:61-72).
__device__ void build_root(uint8_t* sb, const Lay& L, int lane)
{
    uint4 z = make_uint4(0, 0, 0, 0);
    for (int q = lane; q < (L.sbytes >> 4); q += 32) reinterpret_cast<uint4*>(sb)[q] = z;
    __syncwarp();
    for (int j = lane; j < L.n; j += 32) RD(sb, L)[j] = (uint8_t)j;
    if (lane == 0) {
        *H_R(sb, L) = (uint16_t)L.n;
        *H_NS(sb, L) = 0;
        *H_CMAX(sb, L) = 0;
        *H_LIN(sb, L) = kMark;
        *H_STAMP(sb, L) = 0;
    }
    __syncwarp();
}

// Ready ops of the state in `sb`, lane-major: position i = lane + 32*q, q < NQ = ceil(n/32).
template <int NQ>
struct ReadyOps {
    int r;
    int job[NQ], k[NQ], mc[NQ], du[NQ];
};

template <int NQ>
__device__ __forceinline__ void load_ready(uint8_t* sb, const Lay& L, const uint32_t* ops,
                                           int op_off, int lane, ReadyOps<NQ>& R)
{
    R.r = *H_R(sb, L);
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        int i = lane + 32 * q;
        R.mc[q] = -1;
        R.job[q] = 0;
        R.k[q] = 0;
        R.du[q] = 0;
        if (i < R.r) {
            int j = RD(sb, L)[i];
            int k = NX(sb, L)[j];
            uint32_t o = op_info(ops, op_off, j, L.m, k);
            R.job[q] = j;
            R.k[q] = k;
            R.mc[q] = (int)(o & 0xFFu);
            R.du[q] = (int)(o >> 8);
        }
    }
}

// Pivot machine and candidate ballot (gpu/v1/solver.cu:47-69): thread 0 of the reference
// hashes (seed + rank), takes that ready op's machine, and lists the ready ops on that
// machine in ready-list order; here every lane tests its ops and a ballot gives each
// candidate its branch index b.
template <int NQ>
struct Cands {
    unsigned bal[NQ];
    int bidx[NQ];
    int cnt;
    int pm;
};

template <int NQ>
__device__ __forceinline__ void pivot_candidates(const ReadyOps<NQ>& R, uint32_t seed_t, uint32_t c,
                                                 int lane, Cands<NQ>& C)
{
    C.cnt = 0;
    C.pm = -1;
#pragma unroll
    for (int q = 0; q < NQ; q++) { C.bal[q] = 0; C.bidx[q] = 0; }
    if (R.r <= 0) return;
    uint32_t h = pivot_hash(seed_t + c);
    int pp = (int)(h % (uint32_t)R.r);
    int qp = pp >> 5;
    int mine = R.mc[0];
#pragma unroll
    for (int q = 1; q < NQ; q++) if (qp == q) mine = R.mc[q];
    int pm = __shfl_sync(FULL_MASK, mine, pp & 31);
    unsigned lt = (1u << lane) - 1u;
    int acc = 0;
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        C.bal[q] = __ballot_sync(FULL_MASK, (lane + 32 * q < R.r) && R.mc[q] == pm);
        C.bidx[q] = acc + __popc(C.bal[q] & lt);
        acc += __popc(C.bal[q]);
    }
    C.cnt = acc;
    C.pm = pm;
}

// Job-predecessor finish of op (job j, step k): jssp_types.h:82 / gpu_snapshot.cuh:58
// read op_finish[op-1] unless op % m == 1.  For m >= 2 that is "job j's previous op, or 0
// for its first op"; for m == 1 the test never holds and op-1 is job j-1's op.
__device__ __forceinline__ int pred_finish(uint8_t* sb, const Lay& L, int j, int k)
{
    if (L.m == 1) return j > 0 ? JR(sb, L)[j - 1] : 0;
    return k == 0 ? 0 : JR(sb, L)[j];
}

// Apply "schedule the ready op at position i" to the state in `b` (warp-collective):
// removal from the ready list (swap-with-last for the gpu modes, gpu/v1/solver.cu:100-106;
// order-preserving erase for ICH/PMS, cpu/v0_ich/solver.cpp:29, cpu/v1_pms/solver.cpp:44-46),
// then dev_schedule_operation (gpu_snapshot.cuh:47-70) and the makespan.
template <int NQ>
__device__ void apply_child(uint8_t* b, const Lay& L, const uint32_t* ops, int op_off, int i,
                            bool erase, uint32_t lineage, uint32_t stamp, int lane)
{
    const int r = *H_R(b, L);
    const int j = RD(b, L)[i];
    const int k = NX(b, L)[j];
    const uint32_t o = op_info(ops, op_off, j, L.m, k);
    const int mc = (int)(o & 0xFFu);
    const int pred = pred_finish(b, L, j, k);
    const int tr = TR(b)[mc];
    const int fin = (tr > pred ? tr : pred) + (int)(o >> 8);
    __syncwarp();
    if (erase) {
        uint8_t v[NQ];
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            int t = lane + 32 * q;
            v[q] = (t >= i && t < r - 1) ? RD(b, L)[t + 1] : 0;
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            int t = lane + 32 * q;
            if (t >= i && t < r - 1) RD(b, L)[t] = v[q];
        }
        __syncwarp();
    }
    // the edits touch distinct bytes: one lane each
    const uint8_t last = RD(b, L)[r - 1];
    const int ns = *H_NS(b, L), cm = *H_CMAX(b, L);
    const bool cont = (k + 1 < L.m);
    __syncwarp();
    if (lane == 0) TR(b)[mc] = fin;
    if (lane == 1) JR(b, L)[j] = fin;
    if (lane == 2 && !erase && i != r - 1) RD(b, L)[i] = last;
    if (lane == 3 && cont) RD(b, L)[r - 1] = (uint8_t)j;
    if (lane == 4) NX(b, L)[j] = (uint8_t)(k + 1);
    if (lane == 5)
        *reinterpret_cast<uint32_t*>(b + L.off_hdr) = ((uint32_t)(ns + 1) << 16) | (uint32_t)(r - 1 + (cont ? 1 : 0));
    if (lane == 6) *H_CMAX(b, L) = cm > fin ? cm : fin;
    if (lane == 7) *H_LIN(b, L) = lineage;
    if (lane == 8) *H_STAMP(b, L) = stamp;
    __syncwarp();
}

// ------------------------------------------------------------------------------------
// Expansion of one state for level t (gpu modes): kernel_expand_beam_layer /
// kernel_score_candidates (gpu/v1/solver.cu:72-127, v2 :68-123) without the per-thread
// snapshot copy -- a child's makespan needs only tr[pivot machine], the job's
// predecessor finish and the parent makespan.  Keys go to this CTA's chunk region at
// positions reserved with a shared-memory counter.
// ------------------------------------------------------------------------------------
template <int NQ, bool SMEM_NOISE>
__device__ void expand_gpu(uint8_t* sb, uint8_t* cb, const Lay& L, const SegDesc& d, SegState& st,
                           const StepArgs& a, int c, int t, int lane, unsigned long long* kstage,
                           int* nv_out, const float* s_noise)
{
    ReadyOps<NQ> R;
    load_ready<NQ>(sb, L, a.ops, d.op_off, lane, R);
    const uint32_t seed_t = d.seed + (uint32_t)t;
    Cands<NQ> C;
    pivot_candidates<NQ>(R, seed_t, (uint32_t)c, lane, C);
    const int ns1 = *H_NS(sb, L) + 1;
    const int pcmax = *H_CMAX(sb, L);
    const int bound = st.bound;
    const int trp = (C.pm >= 0) ? TR(sb)[C.pm] : 0;
    const bool last = (t == d.N - 1);
    const float fns = __int2float_rn(ns1);

    unsigned long long key[NQ];
    unsigned vb[NQ];
    // scored-branch mask words of this parent (b < n <= 128), kept in registers: a
    // dynamically indexed array would live in local memory
    uint32_t wacc0 = 0u, wacc1 = 0u, wacc2 = 0u, wacc3 = 0u;
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        bool valid = false;
        key[q] = 0ull;
        if ((C.bal[q] >> lane) & 1u) {
            const int pred = pred_finish(sb, L, R.job[q], R.k[q]);
            const int fin = (trp > pred ? trp : pred) + R.du[q];
            const int cm = pcmax > fin ? pcmax : fin;
            valid = cm < bound;   // gpu/v1/solver.cu:120
            if (valid) {
                const int b = C.bidx[q];
                // (float)cmax / (float)ns + (float)(h % 1000) / 1e9f, IEEE round-to-nearest;
                // the second quotient comes from a table of its 1000 possible values
                const float base = __fdiv_rn(__int2float_rn(cm), fns);
                const uint32_t ni = noise_hash(seed_t, (uint32_t)c, (uint32_t)b) % 1000u;
                const float sc = __fadd_rn(base, SMEM_NOISE ? s_noise[ni] : __ldg(s_noise + ni));
                const uint32_t slot = (uint32_t)(c * L.n + b);
                key[q] = ((unsigned long long)__float_as_uint(sc) << 32) | slot;
                const uint32_t bit = 1u << (b & 31);
                const int w = b >> 5;
                wacc0 |= (w == 0) ? bit : 0u;
                wacc1 |= (w == 1) ? bit : 0u;
                wacc2 |= (w == 2) ? bit : 0u;
                wacc3 |= (w == 3) ? bit : 0u;
                if (last && ns1 == d.N) {
                    atomicMin(&st.best, ((unsigned long long)(uint32_t)cm << 32) |
                                            ((unsigned long long)slot << 8) | (uint32_t)R.job[q]);
                    atomicMin(a.group_best + d.group, cm);
                }
            }
        }
        vb[q] = __ballot_sync(FULL_MASK, valid);
    }
    int nv = 0;
#pragma unroll
    for (int q = 0; q < NQ; q++) nv += __popc(vb[q]);
    // keys of this parent in branch order: position among the valid ones = popc below,
    // and branch order == ready-list order == lane-major order here
    const unsigned lt = (1u << lane) - 1u;
    int acc = 0;
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        if ((vb[q] >> lane) & 1u) kstage[acc + __popc(vb[q] & lt)] = key[q];
        acc += __popc(vb[q]);
    }
    if (lane == 0) *nv_out = nv;
    if ((d.mode == MODE_V2 || d.mode == MODE_CLEAN) && t < d.N - 1) {
        // branch b -> ready position of its op, read by the next level's materialisation
        uint8_t* row = a.pos_pool + d.pos_off[t & 1] + (int64_t)c * L.n;
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            const int i = lane + 32 * q;
            if ((C.bal[q] >> lane) & 1u) row[C.bidx[q]] = (uint8_t)i;
            if (i >= C.cnt && i < L.n) row[i] = 0xFFu;
        }
    }
#pragma unroll
    for (int w = 0; w < NQ; w++) {
        if (w < d.words) {
            const uint32_t mine = w == 0 ? wacc0 : (w == 1 ? wacc1 : (w == 2 ? wacc2 : wacc3));
            uint32_t word = __reduce_or_sync(FULL_MASK, mine);
            if (lane == 0) a.masks[d.mask_off + (int64_t)c * d.words + w] = word;
        }
    }

    if (d.mode == MODE_V1 && nv > 0) {
        // kernel_expand_beam_layer also writes every scored child's snapshot into its
        // slot c*n+b (gpu/v1/solver.cu:129-145); slots it skips keep older content.
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            unsigned bits = vb[q];
            while (bits) {
                const int l = __ffs(bits) - 1;
                bits &= bits - 1u;
                const int i = 32 * q + l;
                const int b = __shfl_sync(FULL_MASK, C.bidx[q], l);
                const int j = __shfl_sync(FULL_MASK, R.job[q], l);
                warp_copy_smem(cb, sb, L.sbytes, lane);
                __syncwarp();
                apply_child<NQ>(cb, L, a.ops, d.op_off, i, false, ((uint32_t)c << 8) | (uint32_t)j,
                                (uint32_t)(t + 1), lane);
                warp_store(a.slot_pool + d.slot_off + (int64_t)(c * L.n + b) * L.sbytes, cb, L.sbytes, lane);
                __syncwarp();
            }
        }
    }
}

// ICH / PMS: per ready position, the child's makespan, machine and job; the ordered
// serial part (rand() draws, heap) runs in k_heap (cpu/v0_ich/solver.cpp:22-39,
// cpu/v1_pms/solver.cpp:26-62).
template <int NQ>
__device__ void expand_compat(uint8_t* sb, const Lay& L, const SegDesc& d, const StepArgs& a,
                              int c, int lane)
{
    ReadyOps<NQ> R;
    load_ready<NQ>(sb, L, a.ops, d.op_off, lane, R);
    const int pcmax = *H_CMAX(sb, L);
    uint8_t* base = a.aux_pool + d.aux_off + (int64_t)c * d.auxbytes;
    int32_t* cc = reinterpret_cast<int32_t*>(base + 4);
    uint8_t* cmv = base + 4 + 4 * L.n;
    uint8_t* jb = base + 4 + 5 * L.n;
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        int i = lane + 32 * q;
        if (i < R.r) {
            const int pred = pred_finish(sb, L, R.job[q], R.k[q]);
            const int tr = TR(sb)[R.mc[q]];
            const int fin = (tr > pred ? tr : pred) + R.du[q];
            cc[i] = pcmax > fin ? pcmax : fin;
            cmv[i] = (uint8_t)R.mc[q];
            jb[i] = (uint8_t)R.job[q];
        }
    }
    if (lane == 0) *reinterpret_cast<uint32_t*>(base) = (uint32_t)R.r;
}

// ------------------------------------------------------------------------------------
// k_step: materialise level s+1 and expand it.  Work unit: a chunk of CH consecutive
// ranks of one beam per CTA (CH / 8 per warp; CH = a.chunk, chosen per plan).  Each warp first fetches the
// selection entries of its ranks, then starts asynchronous copies of all their source
// snapshots into shared memory, then materialises and expands them one after the other,
// so the copies of later ranks overlap the work on earlier ones.  NQ = ceil(n/32).
// ------------------------------------------------------------------------------------
template <int NQ, int CH>
#ifndef BSJ_STEP_MIN_BLOCKS
#define BSJ_STEP_MIN_BLOCKS 4
#endif
#ifndef BSJ_STEP_MIN_BLOCKS_WIDE
#define BSJ_STEP_MIN_BLOCKS_WIDE 6
#endif
// Resident CTAs per SM (register budget): four (64 registers) by default, three for
// n > 64.  For 33 <= n <= 64 the 16- and 32-survivor chunks -- which the chunk rule picks
// for wide levels, where the GPU's k_step throughput bounds a level -- take six (42
// registers): 37.0 vs 38.1 ms on 8 beams x K=4096 at 50x20; the 8-survivor chunk, picked
// for narrow latency-bound levels, keeps four (six cost a single such beam 4-5 %).
__global__ void __launch_bounds__(kWarpsPerStepCta * 32,
                                  NQ == 4 ? 3 : (NQ == 2 && CH >= 16) ? BSJ_STEP_MIN_BLOCKS_WIDE : BSJ_STEP_MIN_BLOCKS)
k_step(StepArgs a, int s)
{
    constexpr int kRanksPerWarp = CH / kWarpsPerStepCta;
    extern __shared__ __align__(16) uint8_t smem[];
    // noise quotients: small chunks read the plan's table through L1, 32-survivor chunks
    // (more candidates per CTA) copy it into shared memory once
    __shared__ float s_noise_tab[CH >= 32 ? 1000 : 1];
    __shared__ int s_nv[CH], s_pre[CH], s_kcnt, s_P;
    __shared__ uint32_t s_mm[2];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint8_t* wbuf = smem + (size_t)warp * (kRanksPerWarp + 1) * a.sb_max;
    uint8_t* cb = wbuf + (size_t)kRanksPerWarp * a.sb_max;
    // candidate keys of the chunk's ranks, staged per rank (n slots each) so that they
    // leave in slot order: ranks ascending, branches ascending
    unsigned long long* kstage = reinterpret_cast<unsigned long long*>(
        smem + (size_t)kWarpsPerStepCta * (kRanksPerWarp + 1) * a.sb_max);
    pdl_trigger();
    if constexpr (CH >= 32)
        for (int k = threadIdx.x; k < 1000; k += blockDim.x) s_noise_tab[k] = __ldg(a.noise + k);
    pdl_wait();
    const float* s_noise = CH >= 32 ? s_noise_tab : a.noise;
    for (int chunk = a.chunk_lo + blockIdx.x; chunk < a.chunk_hi; chunk += gridDim.x) {
        const int seg = find_seg(a.chunk_prefix, a.seg_lo, a.seg_hi, chunk);
        const SegDesc& d = a.segs[seg];
        if (d.nq != NQ || s >= d.N - 1) continue;
        SegState& st = a.st[seg];
        const int q = chunk - __ldg(a.chunk_prefix + seg);
        if (threadIdx.x == 0) s_P = (s < 0) ? 1 : *((volatile int32_t*)&st.P);
        if (threadIdx.x < CH) s_nv[threadIdx.x] = 0;
        __syncthreads();
        const int P = s_P;
        const Lay L(d);
        const int mode = d.mode;
        const bool compat = (mode == MODE_ICH || mode == MODE_PMS);
        const int r0 = q * CH + warp;
        uint8_t* childbuf = a.beam_pool + d.beam_off[(s + 1) & 1];
        const uint8_t* parent = a.beam_pool + d.beam_off[s & 1];
        if (mode == MODE_V1) childbuf = a.beam_pool + d.beam_off[0];

        // selection entries of this warp's ranks (one lane each) and, for the gpu modes,
        // the ready-list position of the selected branch's op
        uint32_t my_e = 0, my_pos = 0xFFu;
        if (lane < kRanksPerWarp && s >= 0) {
            const int r = r0 + lane * kWarpsPerStepCta;
            if (r < P && mode != MODE_V1) {
                my_e = __ldg(a.sel + d.sel_off + r);
                if (!compat) my_pos = __ldg(a.pos_pool + d.pos_off[s & 1] + (my_e & ~kFillerFlag));
            }
        }
        // start all source copies
#pragma unroll
        for (int i = 0; i < kRanksPerWarp; i++) {
            const int r = r0 + i * kWarpsPerStepCta;
            const uint32_t e = __shfl_sync(FULL_MASK, my_e, i);
            if (r >= P || s < 0) continue;
            const uint8_t* src;
            if (mode == MODE_V1) src = childbuf + (int64_t)r * L.sbytes;
            else if (compat) src = parent + (int64_t)(e >> 8) * L.sbytes;
            else src = parent + (int64_t)((e & ~kFillerFlag) / (uint32_t)L.n) * L.sbytes;
            warp_prefetch(wbuf + (size_t)i * a.sb_max, src, L.sbytes, lane);
        }
        cp_async_commit();
        cp_async_wait_all();
        __syncwarp();

        unsigned long long* kdst = a.keys + d.key_off + (int64_t)q * CH * L.n;
        const int nst = L.n;  // staged keys per rank
        uint32_t* hrow = a.hist + d.hist_off + (int64_t)(s < 0 ? 0 : s) * d.K;
#pragma unroll 1
        for (int i = 0; i < kRanksPerWarp; i++) {
            const int r = r0 + i * kWarpsPerStepCta;
            if (r >= P) break;
            uint8_t* sb = wbuf + (size_t)i * a.sb_max;
            const uint32_t e = __shfl_sync(FULL_MASK, my_e, i);
            if (s < 0) {
                build_root(sb, L, lane);
                warp_store(childbuf, sb, L.sbytes, lane);
            } else if (compat) {
                const int c = (int)(e >> 8), ii = (int)(e & 0xFFu);
                const int j = RD(sb, L)[ii];
                apply_child<NQ>(sb, L, a.ops, d.op_off, ii, true, ((uint32_t)c << 8) | (uint32_t)j,
                                (uint32_t)(s + 1), lane);
                warp_store(childbuf + (int64_t)r * L.sbytes, sb, L.sbytes, lane);
                if (lane == 0) hrow[r] = ((uint32_t)c << 8) | (uint32_t)j;
            } else if (mode != MODE_V1) {
                const uint32_t slot = e & ~kFillerFlag;
                const int c = (int)(slot / (uint32_t)L.n);
                const int ii = (int)__shfl_sync(FULL_MASK, my_pos, i);
                if (ii != 0xFF) {
                    // kernel_materialize_topk (gpu/v2_twophases/solver.cu:193-252): the
                    // parent's expansion recorded where branch b's op sits in its ready list
                    const int j = RD(sb, L)[ii];
                    apply_child<NQ>(sb, L, a.ops, d.op_off, ii, false, ((uint32_t)c << 8) | (uint32_t)j,
                                    (uint32_t)(s + 1), lane);
                    warp_store(childbuf + (int64_t)r * L.sbytes, sb, L.sbytes, lane);
                    if (lane == 0) hrow[r] = ((uint32_t)c << 8) | (uint32_t)j;
                } else {
                    // filler rank: v2 leaves the ping-pong slot as it was (:191)
                    if (mode == MODE_CLEAN && lane == 0) atomicOr(&st.status, kStatusBadSelect);
                    __syncwarp();
                    warp_load(sb, childbuf + (int64_t)r * L.sbytes, L.sbytes, lane);
                    if (lane == 0) hrow[r] = kMark;
                }
            }
            __syncwarp();
            if (compat) expand_compat<NQ>(sb, L, d, a, r, lane);
            else {
                const int rl = r - q * CH;
                expand_gpu<NQ, (CH >= 32)>(sb, cb, L, d, st, a, r, s + 1, lane, kstage + (size_t)rl * nst, &s_nv[rl],
                                           s_noise);
            }
        }
        __syncthreads();
        if (!compat) {
            // rank-ordered prefix of the staged counts, then coalesced copy-out
            if (warp == 0) {
                const int v = lane < CH ? s_nv[lane] : 0;
                int x = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(FULL_MASK, x, o);
                    if (lane >= o) x += y;
                }
                if (lane < CH) s_pre[lane] = x - v;
                if (lane == 31) s_kcnt = x;
                if (lane == 0) { s_mm[0] = 0xFFFFFFFFu; s_mm[1] = 0u; }
            }
            __syncthreads();
            uint32_t mn = 0xFFFFFFFFu, mx = 0u;
            for (int rl = warp; rl < CH; rl += kWarpsPerStepCta) {
                const int cntk = s_nv[rl];
                const int dst0 = s_pre[rl];
                for (int i = lane; i < cntk; i += 32) {
                    const unsigned long long k = kstage[(size_t)rl * nst + i];
                    kdst[dst0 + i] = k;
                    mn = min(mn, (uint32_t)(k >> 32));
                    mx = max(mx, (uint32_t)(k >> 32));
                }
            }
            chunk_range_add(mn, mx, s_mm, lane);
        }
        __syncthreads();
        if (!compat && threadIdx.x == 0) {
            a.kcnt[d.kcnt_off + q] = s_kcnt;
            a.kmm[d.kcnt_off + q] = make_uint2(s_mm[0], s_mm[1]);
        }
    }
}

// ------------------------------------------------------------------------------------
// k_gather_v1: kernel_gather_topk (gpu/v1/solver.cu:160-176), warp per survivor, 16-byte
// vector copies.
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kWarpsPerStepCta * 32) k_gather_v1(StepArgs a, int s)
{
    pdl_wait();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nw = gridDim.x * kWarpsPerStepCta;
    for (int flat = a.rank_lo + blockIdx.x * kWarpsPerStepCta + warp; flat < a.rank_hi; flat += nw) {
        const int seg = find_seg(a.rank_prefix, a.seg_lo, a.seg_hi, flat);
        const SegDesc& d = a.segs[seg];
        if (d.mode != MODE_V1 || s >= d.N - 1) continue;
        const int r = flat - __ldg(a.rank_prefix + seg);
        if (r >= a.st[seg].P) continue;
        const uint32_t slot = __ldg(a.sel + d.sel_off + r) & ~kFillerFlag;
        const uint8_t* src = a.slot_pool + d.slot_off + (int64_t)slot * d.sbytes;
        uint8_t* dst = a.beam_pool + d.beam_off[0] + (int64_t)r * d.sbytes;
        const uint4* s4 = reinterpret_cast<const uint4*>(src);
        uint4* d4 = reinterpret_cast<uint4*>(dst);
        for (int q = lane; q < (d.sbytes >> 4); q += 32) d4[q] = s4[q];
        if (lane == 0) {
            const uint32_t lin = *reinterpret_cast<const uint32_t*>(src + d.off_hdr + 8);
            const uint32_t stamp = *reinterpret_cast<const uint32_t*>(src + d.off_hdr + 12);
            a.hist[d.hist_off + (int64_t)s * d.K + r] = (stamp == (uint32_t)(s + 1)) ? lin : kMark;
        }
    }
}

// ------------------------------------------------------------------------------------
// Helpers of the lane-group k_step below: one survivor's snapshot in shared memory read
// and written field by field, and the beam's layout held in registers.
// ------------------------------------------------------------------------------------
constexpr uint32_t kTSpinLimit = 1u << 22;     // mbarrier try_wait attempts before giving up

// One lane's snapshot in shared memory: word x at w[x * XS].
template <int XS>
struct TSnap {
    uint32_t* w;
    __device__ __forceinline__ uint32_t word(int x) const { return w[x * XS]; }
    __device__ __forceinline__ void set_word(int x, uint32_t v) const { w[x * XS] = v; }
    __device__ __forceinline__ int byte(int off) const { return (int)((w[(off >> 2) * XS] >> ((off & 3) * 8)) & 0xFFu); }
    __device__ __forceinline__ void set_byte(int off, int v) const
    {
        reinterpret_cast<uint8_t*>(w + (off >> 2) * XS)[off & 3] = (uint8_t)v;
    }
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// The snapshot layout and instance of one beam, in registers (the kernel writes global
// memory inside its loops, so fields read through a SegDesc reference would be reloaded).
struct TLay {
    int n, m, N, sbytes, off_jr4, off_rd, off_nx, hw;
    const uint32_t* ops;   // this instance's (duration << 8) | machine table
    __device__ __forceinline__ TLay(const SegDesc& d, const uint32_t* all_ops)
        : n(d.n), m(d.m), N(d.N), sbytes(d.sbytes), off_jr4(d.off_jr >> 2), off_rd(d.off_rd),
          off_nx(d.off_nx), hw(d.off_hdr >> 2), ops(all_ops + d.op_off) {}
    __device__ __forceinline__ uint32_t op(int j, int k) const { return __ldg(ops + j * m + k); }
};

// Job-predecessor finish (pred_finish above, on a lane's snapshot).
template <int XS>
__device__ __forceinline__ int tpred_finish(const TSnap<XS>& S, const TLay& L, int j, int k)
{
    if (L.m == 1) return j > 0 ? (int)S.word(L.off_jr4 + j - 1) : 0;
    return k == 0 ? 0 : (int)S.word(L.off_jr4 + j);
}

// Ready position of the b-th candidate of the expansion of this (parent) snapshot at
// level t as rank c -- the pivot machine's ready ops in ready-list order -- or -1 when the
// parent has at most b candidates.  Only filler ranks need it (a scored child's position
// comes from the table its parent's expansion wrote).
template <int XS>
__device__ int tnth_candidate(const TSnap<XS>& S, const TLay& L, uint32_t seed_t, int c, int b)
{
    const int rr = (int)(S.word(L.hw) & 0xFFFFu);
    if (rr <= 0) return -1;
    const uint32_t h = pivot_hash(seed_t + (uint32_t)c);
    const int jp = S.byte(L.off_rd + (int)(h % (uint32_t)rr));
    const int pm = (int)(L.op(jp, S.byte(L.off_nx + jp)) & 0xFFu);
    int cnt = 0;
    for (int i = 0; i < rr; i++) {
        const int j = S.byte(L.off_rd + i);
        if ((int)(L.op(j, S.byte(L.off_nx + j)) & 0xFFu) == pm) {
            if (cnt == b) return i;
            cnt++;
        }
    }
    return -1;
}

// ------------------------------------------------------------------------------------
// k_step_g: materialise + expand with a GROUP of G lanes per survivor (gpu-v2 / clean
// beams), 32/G survivors per warp, 4 warps per CTA: CH = 128/G consecutive ranks per CTA
// (one key chunk of CH).  Between the warp form (every lane on one survivor: most lanes
// idle) and the thread form (one lane per survivor: a long serial chain per lane), the
// group splits what is long -- staging the parent, storing the child, scanning the ready
// list -- and keeps what is short on the group's first lane (applying the selected op).
// Candidates are numbered in ready-list order with group-masked ballots, scored by the
// lane that found them and staged per survivor in shared memory; the CTA copies its
// chunk's keys out in slot order.
// Staging of the parent snapshot (template STG): 1 = 16-byte cp.async by the group's lanes;
// 2 = one cp.async.bulk (TMA bulk copy) per survivor issued by the group's first lane,
// completing on a per-warp mbarrier.
// Result-identical to k_step (same arithmetic in the same order per child).
// ------------------------------------------------------------------------------------
constexpr int kGStepWarps = 4;

__host__ __device__ __forceinline__ size_t gstep_smem_bytes(int G, int sb_max, int max_n)
{
    const size_t ch = (size_t)kGStepWarps * (size_t)(32 / G);
    return ch * (size_t)sb_max + ch * (size_t)max_n * 8;
}

template <int G, int STG>
__global__ void __launch_bounds__(kGStepWarps * 32) k_step_g(StepArgs a, int s)
{
    constexpr int SPW = 32 / G;            // survivors per warp
    constexpr int CH = kGStepWarps * SPW;  // survivors per CTA = key chunk size
    constexpr bool BULK = (STG == 2);
    constexpr unsigned kLowG = (1u << G) - 1u;
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ __align__(8) unsigned long long s_mbar[kGStepWarps];
    __shared__ int s_nv[CH], s_pre[CH], s_kcnt, s_abort;
    __shared__ uint32_t s_mm[2];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grp = lane / G, gl = lane % G, gsh = grp * G;
    const int slot = warp * SPW + grp;
    const unsigned ltg = (1u << gl) - 1u;
    uint8_t* sb = smem + (size_t)slot * a.sb_max;
    unsigned long long* kst =
        reinterpret_cast<unsigned long long*>(smem + (size_t)CH * a.sb_max) + (size_t)slot * a.max_n;
    TSnap<1> S;
    S.w = reinterpret_cast<uint32_t*>(sb);
    pdl_trigger();
    if (BULK) {
        if (lane == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&s_mbar[warp])), "r"(32) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncwarp();
    }
    if (threadIdx.x == 0) s_abort = 0;
    __syncthreads();
    uint32_t phase = 0;
    pdl_wait();
    for (int chunk = a.chunk_lo + blockIdx.x; chunk < a.chunk_hi; chunk += gridDim.x) {
        const int seg = find_seg(a.chunk_prefix, a.seg_lo, a.seg_hi, chunk);
        const SegDesc& d = a.segs[seg];
        if (s >= d.N - 1) continue;   // the same for the whole CTA (one chunk)
        SegState& st = a.st[seg];
        if (d.mode != MODE_V2 && d.mode != MODE_CLEAN) {   // the host runs only these beams here
            if (threadIdx.x == 0) atomicOr(&st.status, kStatusBadSelect);
            continue;
        }
        const TLay L(d, a.ops);
        const int mode = d.mode, K = d.K, words = d.words, group = d.group;
        const uint32_t seed = d.seed;
        const int q = chunk - __ldg(a.chunk_prefix + seg);
        const int P = (s < 0) ? 1 : *((volatile int32_t*)&st.P);
        const int n = L.n, m = L.m, w16 = L.sbytes >> 4;
        const int r = q * CH + slot;
        const bool act = r < P;
        uint8_t* childbuf = a.beam_pool + d.beam_off[(s + 1) & 1];
        const uint8_t* parent = a.beam_pool + d.beam_off[s & 1];
        const uint8_t* pos_in = a.pos_pool + d.pos_off[s & 1];
        uint8_t* pos_out = a.pos_pool + d.pos_off[(s + 1) & 1];
        const int bound = st.bound;

        // ---- 1. the source snapshot of this rank
        uint32_t e = 0;
        int c = 0, b = 0, ii = -1;
        if (act && s >= 0) {
            e = __ldg(a.sel + d.sel_off + r);
            const uint32_t sl = e & ~kFillerFlag;
            c = (int)(sl / (uint32_t)n);
            b = (int)sl - c * n;
            if (!(e & kFillerFlag)) ii = __ldg(pos_in + sl);
        }
        const uint8_t* src = parent + (int64_t)c * L.sbytes;
        bool ok = true;
        if (BULK) {
            const uint32_t bar = smem_u32(&s_mbar[warp]);
            if (gl == 0 && act && s >= 0) {
                // the slot was last written through the generic proxy: order that before
                // the bulk copy's (async-proxy) write
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n"
                             ::"r"(bar), "r"(L.sbytes) : "memory");
                asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                             ::"r"(smem_u32(sb)), "l"(src), "r"(L.sbytes), "r"(bar) : "memory");
            } else {
                asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(bar)
                             : "memory");
            }
            uint32_t done = 0;
            for (uint32_t it = 0; it < kTSpinLimit && !done; it++) {
                asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                             " selp.u32 %0, 1, 0, p;\n}\n"
                             : "=r"(done) : "r"(bar), "r"(phase) : "memory");
            }
            phase ^= 1u;
            if (!__all_sync(FULL_MASK, done)) {
                // a copy that never completed: flag it, wait once more (bounded) for the
                // warp's copies, take no part in this chunk and make the CTA stop after it
                // (every warp still reaches the chunk's barriers)
                if (lane == 0) {
                    atomicOr(&st.status, kStatusBadSelect);
                    s_abort = 1;
                }
                for (uint32_t it = 0; it < kTSpinLimit && !done; it++) {
                    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                                 " selp.u32 %0, 1, 0, p;\n}\n"
                                 : "=r"(done) : "r"(bar), "r"(phase ^ 1u) : "memory");
                }
                ok = false;
            }
        } else {
            if (act && s >= 0)
                for (int x = gl; x < w16; x += G) cp_async16(sb + 16 * x, src + 16 * x);
            cp_async_commit();
            cp_async_wait_all();
        }
        __syncwarp();
        const bool live = act && ok;

        // ---- 2. materialise (v2: kernel_materialize_topk, gpu/v2_twophases/solver.cu:193-252)
        // a filler's branch position comes from the parent's expansion, recomputed
        int fii = -1;
        if (gl == 0 && live && s >= 0 && (e & kFillerFlag))
            fii = tnth_candidate<1>(S, L, seed + (uint32_t)s, c, b);
        fii = __shfl_sync(FULL_MASK, fii, gsh);
        if (e & kFillerFlag) ii = fii;
        const bool do_root = live && s < 0;
        const bool do_apply = live && s >= 0 && ii >= 0;
        const bool do_stale = live && s >= 0 && ii < 0;
        uint32_t hist_val = kMark;
        if (gl == 0 && do_root) {
            for (int x = 0; x < (L.sbytes >> 2); x++) S.set_word(x, 0u);
            for (int j = 0; j < n; j++) S.set_byte(L.off_rd + j, j);
            S.set_word(L.hw, (uint32_t)n);
            S.set_word(L.hw + 2, kMark);
        }
        if (gl == 0 && do_apply) {
            const uint32_t h0 = S.word(L.hw);
            const int r0 = (int)(h0 & 0xFFFFu), ns = (int)(h0 >> 16);
            const int j = S.byte(L.off_rd + ii);
            const int k = S.byte(L.off_nx + j);
            const uint32_t o = L.op(j, k);
            const int mc = (int)(o & 0xFFu);
            const int pred = tpred_finish<1>(S, L, j, k);
            const int trv = (int)S.word(mc);
            const int fin = (trv > pred ? trv : pred) + (int)(o >> 8);
            const int lastj = S.byte(L.off_rd + r0 - 1);
            const bool cont = (k + 1 < m);
            const int cm = (int)S.word(L.hw + 1);
            S.set_word(mc, (uint32_t)fin);
            S.set_word(L.off_jr4 + j, (uint32_t)fin);
            if (ii != r0 - 1) S.set_byte(L.off_rd + ii, lastj);
            if (cont) S.set_byte(L.off_rd + r0 - 1, j);
            S.set_byte(L.off_nx + j, k + 1);
            S.set_word(L.hw, ((uint32_t)(ns + 1) << 16) | (uint32_t)(r0 - 1 + (cont ? 1 : 0)));
            S.set_word(L.hw + 1, (uint32_t)(cm > fin ? cm : fin));
            hist_val = ((uint32_t)c << 8) | (uint32_t)j;
            S.set_word(L.hw + 2, hist_val);
            S.set_word(L.hw + 3, (uint32_t)(s + 1));
        }
        if (do_stale) {
            // filler rank whose branch does not exist: v2 leaves the ping-pong slot as it
            // was (gpu/v2_twophases/solver.cu:191) and expands what it holds
            const uint4* s4 = reinterpret_cast<const uint4*>(childbuf + (int64_t)r * L.sbytes);
            for (int x = gl; x < w16; x += G) reinterpret_cast<uint4*>(sb)[x] = __ldcg(s4 + x);
            if (gl == 0 && mode == MODE_CLEAN) atomicOr(&st.status, kStatusBadSelect);
        }
        __syncwarp();
        if (do_root || do_apply) {
            uint4* d4 = reinterpret_cast<uint4*>(childbuf + (int64_t)r * L.sbytes);
            for (int x = gl; x < w16; x += G) d4[x] = reinterpret_cast<const uint4*>(sb)[x];
        }
        if (gl == 0 && live && s >= 0) a.hist[d.hist_off + (int64_t)s * K + r] = hist_val;

        // ---- 3. expand for level t (kernel_score_candidates, gpu/v2_twophases/solver.cu:68-123)
        const int t = s + 1;
        const uint32_t seed_t = seed + (uint32_t)t;
        const bool lastlv = (t == L.N - 1);
        const bool rows = t < L.N - 1;
        const int rr = live ? (int)(S.word(L.hw) & 0xFFFFu) : 0;
        const int rrmax = __reduce_max_sync(FULL_MASK, (unsigned)rr);
        int ns1 = 1, pcmax = 0, trp = 0, pm = -1;
        if (rr > 0) {
            const uint32_t h0 = S.word(L.hw);
            ns1 = (int)(h0 >> 16) + 1;
            pcmax = (int)S.word(L.hw + 1);
            const uint32_t h = pivot_hash(seed_t + (uint32_t)r);
            const int jp = S.byte(L.off_rd + (int)(h % (uint32_t)rr));
            pm = (int)(L.op(jp, S.byte(L.off_nx + jp)) & 0xFFu);
            trp = (int)S.word(pm);
        }
        const float fns = __int2float_rn(ns1);
        uint8_t* prow = pos_out + (int64_t)r * n;
        int carry = 0, vcarry = 0;
        uint32_t vm0 = 0u, vm1 = 0u, vm2 = 0u, vm3 = 0u;
        for (int i0 = 0; i0 < rrmax; i0 += G) {
            const int i = i0 + gl;
            bool on = false, valid = false;
            int j = 0, cmx = 0;
            if (i < rr) {
                j = S.byte(L.off_rd + i);
                const int k = S.byte(L.off_nx + j);
                const uint32_t o = L.op(j, k);
                on = (int)(o & 0xFFu) == pm;
                if (on) {
                    const int pred = tpred_finish<1>(S, L, j, k);
                    const int fin = (trp > pred ? trp : pred) + (int)(o >> 8);
                    cmx = pcmax > fin ? pcmax : fin;
                    valid = cmx < bound;   // gpu/v1/solver.cu:120
                }
            }
            const unsigned gb = (__ballot_sync(FULL_MASK, on) >> gsh) & kLowG;
            const unsigned gv = (__ballot_sync(FULL_MASK, valid) >> gsh) & kLowG;
            if (on) {
                const int bidx = carry + __popc(gb & ltg);
                if (rows) prow[bidx] = (uint8_t)i;
                if (valid) {
                    const int vidx = vcarry + __popc(gv & ltg);
                    const float base = __fdiv_rn(__int2float_rn(cmx), fns);
                    const uint32_t ni = noise_hash(seed_t, (uint32_t)r, (uint32_t)bidx) % 1000u;
                    const float sc = __fadd_rn(base, __ldg(a.noise + ni));
                    const uint32_t sl = (uint32_t)(r * n + bidx);
                    kst[vidx] = ((unsigned long long)__float_as_uint(sc) << 32) | sl;
                    const uint32_t bit = 1u << (bidx & 31);
                    const int wq = bidx >> 5;
                    vm0 |= (wq == 0) ? bit : 0u;
                    vm1 |= (wq == 1) ? bit : 0u;
                    vm2 |= (wq == 2) ? bit : 0u;
                    vm3 |= (wq == 3) ? bit : 0u;
                    if (lastlv && ns1 == L.N) {
                        atomicMin(&st.best, ((unsigned long long)(uint32_t)cmx << 32) |
                                                ((unsigned long long)sl << 8) | (uint32_t)j);
                        atomicMin(a.group_best + group, cmx);
                    }
                }
            }
            carry += __popc(gb);
            vcarry += __popc(gv);
        }
        // the group's scored-branch mask words (lanes of a group differ in their low bits)
#pragma unroll
        for (int o = 1; o < G; o <<= 1) {
            vm0 |= __shfl_xor_sync(FULL_MASK, vm0, o);
            vm1 |= __shfl_xor_sync(FULL_MASK, vm1, o);
            vm2 |= __shfl_xor_sync(FULL_MASK, vm2, o);
            vm3 |= __shfl_xor_sync(FULL_MASK, vm3, o);
        }
        if (gl == 0) {
            s_nv[slot] = live ? vcarry : 0;
            if (live) {
#pragma unroll
                for (int w = 0; w < 4; w++)
                    if (w < words)
                        a.masks[d.mask_off + (int64_t)r * words + w] =
                            w == 0 ? vm0 : (w == 1 ? vm1 : (w == 2 ? vm2 : vm3));
            }
        }
        __syncthreads();
        // ---- 4. the chunk's keys out in slot order
        if (warp == 0) {
            const int v = lane < CH ? s_nv[lane] : 0;
            int x = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(FULL_MASK, x, o);
                if (lane >= o) x += y;
            }
            if (lane < CH) s_pre[lane] = x - v;
            if (lane == 31) s_kcnt = x;
            if (lane == 0) { s_mm[0] = 0xFFFFFFFFu; s_mm[1] = 0u; }
        }
        __syncthreads();
        unsigned long long* kdst = a.keys + d.key_off + (int64_t)q * CH * n;
        uint32_t mn = 0xFFFFFFFFu, mx = 0u;
        for (int rl = warp; rl < CH; rl += kGStepWarps) {
            const int cntk = s_nv[rl], dst0 = s_pre[rl];
            const unsigned long long* ks =
                reinterpret_cast<const unsigned long long*>(smem + (size_t)CH * a.sb_max) + (size_t)rl * a.max_n;
            for (int x = lane; x < cntk; x += 32) {
                const unsigned long long k = ks[x];
                kdst[dst0 + x] = k;
                mn = min(mn, (uint32_t)(k >> 32));
                mx = max(mx, (uint32_t)(k >> 32));
            }
        }
        chunk_range_add(mn, mx, s_mm, lane);
        __syncthreads();
        if (threadIdx.x == 0) {
            a.kcnt[d.kcnt_off + q] = s_kcnt;
            a.kmm[d.kcnt_off + q] = make_uint2(s_mm[0], s_mm[1]);
        }
        if (s_abort) break;
    }
}

// ------------------------------------------------------------------------------------
// k_select: exact top-K + stable order per beam (gpu modes).
//
// The reference sorts all P*n (score, slot) pairs with a stable radix sort and keeps the
// first min(P*n, K) (gpu/v1/solver.cu:255-274).  Scores of skipped slots are 1e9f, above
// every real score, so the kept list is: the real candidates in ascending
// (score bits, slot) order, then -- only when fewer than min(P*n,K) are real -- the
// lowest-numbered skipped slots ("fillers").  Keys are unique 64-bit
// (score bits << 32 | slot), so the top-K set is exact: an MSD radix select finds the
// K-th key, survivors are compacted and bitonic-sorted in shared memory.
// ------------------------------------------------------------------------------------
struct SelSmem {
    uint32_t* hist;            // 16 KB: u32[4096] bucket counts | u16[32][256] digit counters | u32[16][256]
    uint32_t* tot;             // [256]
    unsigned long long* red;   // [64]
    int* misc;                 // [64]
    unsigned long long* A;     // [kLsdMax]   compacted survivors / radix-sort buffer
    unsigned long long* stg;   // [kStageKeys] staged candidate keys / radix-sort buffer / wide bitonic
    uint32_t rmin, rmax;       // min / max score bits of the level's keys (from k_step's chunk ranges)
};

constexpr int kLsdMax = 8192;      // largest survivor count for the radix sort
constexpr int kStageKeys = 16384;  // candidate keys staged in shared memory

__device__ __forceinline__ SelSmem sel_smem(uint8_t* base, uint32_t rmin = 0xFFFFFFFFu, uint32_t rmax = 0u)
{
    SelSmem s;
    s.rmin = rmin;
    s.rmax = rmax;
    s.hist = reinterpret_cast<uint32_t*>(base);
    s.tot = s.hist + 4096;
    s.red = reinterpret_cast<unsigned long long*>(s.tot + 256);
    s.misc = reinterpret_cast<int*>(s.red + 64);
    s.A = reinterpret_cast<unsigned long long*>(s.misc + 64);
    s.stg = s.A + kLsdMax;
    return s;
}

size_t select_smem_bytes(int)
{
    return (size_t)(4096 + 256) * 4 + 64 * 8 + 64 * 4 + (size_t)(kLsdMax + kStageKeys) * 8;
}

// Block-wide exclusive scan of one int per thread; returns the prefix, *total the sum.
__device__ int block_exclusive_scan(int v, int* total, int* warp_sums)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(FULL_MASK, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nwarps ? warp_sums[lane] : 0;
        int ws = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(FULL_MASK, ws, o);
            if (lane >= o) ws += y;
        }
        warp_sums[32 + lane] = ws - w;
        if (lane == 31) warp_sums[64] = ws;
    }
    __syncthreads();
    int res = warp_sums[32 + warp] + x - v;
    *total = warp_sums[64];
    __syncthreads();
    return res;
}

// Candidate keys of one beam live in per-chunk regions of cap keys each, filled to
// cpref[c+1]-cpref[c]; logical key i is found by a binary search over the prefix.
struct KeySrc {
    const unsigned long long* base;
    const int* cpref;  // shared memory, nch+1 entries
    int nch;
    int cap;
    __device__ __forceinline__ unsigned long long operator()(int i) const
    {
        int lo = 0, hi = nch;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (cpref[mid] <= i) lo = mid; else hi = mid;
        }
        return base[(size_t)lo * cap + (i - cpref[lo])];
    }
    // fn(key) on every key, warp per chunk (order not preserved)
    template <typename Fn>
    __device__ __forceinline__ void each_key(Fn fn) const
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int c = warp; c < nch; c += nw) {
            const int c0 = cpref[c], nc = cpref[c + 1] - c0;
            const unsigned long long* src = base + (size_t)c * cap;
            for (int j = lane; j < nc; j += 32) fn(src[j]);
        }
    }
    // keys i0 .. i0+KPT-1 (~0 past V): one search, then walk the chunks
    template <int KPT>
    __device__ __forceinline__ void load_run(int i0, int V, unsigned long long (&out)[KPT]) const
    {
        int lo = 0, hi = nch;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (cpref[mid] <= i0) lo = mid; else hi = mid;
        }
#pragma unroll
        for (int q = 0; q < KPT; q++) {
            const int i = i0 + q;
            if (i < V) {
                while (lo + 1 < nch && cpref[lo + 1] <= i) lo++;
                out[q] = base[(size_t)lo * cap + (i - cpref[lo])];
            } else {
                out[q] = ~0ull;
            }
        }
    }
};

// ---- top-K selection -----------------------------------------------------------------
// 1. stage: the level's candidate keys (slot order) into shared memory, coalesced.
// 2. threshold: one histogram pass over 4096 linear buckets of the score bits gives the
//    bucket T holding rank R; every key of buckets <= T is kept (R plus the rest of T).
//    If that set is too large, MSD radix passes over the 64-bit keys find the R-th key
//    exactly instead.
// 3. compact the kept keys, stably (slot order preserved), with one block scan.
// 4. stable LSD radix sort by the score bits only -- the input is in slot order, so this
//    is exactly the reference's stable (score, slot) order -- and emit the first R.
constexpr int kNB = 4096;

__device__ __forceinline__ unsigned long long umin64(unsigned long long a, unsigned long long b) { return a < b ? a : b; }
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) { return a < b ? b : a; }

__device__ __forceinline__ int pow2ceil(int c)
{
    return c <= 1 ? 1 : 1 << (32 - __clz(c - 1));
}

__device__ __forceinline__ void cp_async8(void* smem_dst, const void* gmem_src)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem_src) : "memory");
}

// 1. all V keys, logical order, into stg (warp per chunk, consecutive lanes -> consecutive keys)
__device__ void stage_keys(const KeySrc& ks, unsigned long long* stg)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int c = warp; c < ks.nch; c += nwarps) {
        const int c0 = ks.cpref[c], nc = ks.cpref[c + 1] - c0;
        const unsigned long long* src = ks.base + (size_t)c * ks.cap;
        for (int i = lane; i < nc; i += 32) cp_async8(stg + c0 + i, src + i);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();
}

// Bucket of a score (bits) in [smin, smin + 4096 << shift); clamped, so a score outside the
// recorded range cannot index past the counts.
__device__ __forceinline__ uint32_t bucket_of(uint32_t sb, uint32_t smin, int shift)
{
    const uint32_t b = (sb - smin) >> shift;
    return b < (uint32_t)kNB ? b : (uint32_t)(kNB - 1);
}

// 2a. bucket threshold over 4096 linear buckets of the score bits between the level's
// min and max (S.rmin / S.rmax): returns the number of keys in buckets <= T; misc[2] = T,
// misc[4] = shift, misc[1] = smin.
// `each(fn)` calls fn on every key this thread is responsible for.
template <typename ForEach>
__device__ int bucket_threshold_each(ForEach each, int R, const SelSmem& S)
{
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31;
    uint32_t* cnt = S.hist;
    int* misc = S.misc;
    int* wsum = reinterpret_cast<int*>(S.red);
    (void)lane;
    for (int b = tid; b < kNB; b += nthr) cnt[b] = 0;
    if (tid == 0) misc[1] = (int)S.rmin;
    __syncthreads();
    const uint32_t smin = S.rmin, range = S.rmax - S.rmin;
    const int nbits = range ? 32 - __clz(range) : 0;
    const int shift = nbits > 12 ? nbits - 12 : 0;
    each([&](unsigned long long k) { atomicAdd(&cnt[bucket_of((uint32_t)(k >> 32), smin, shift)], 1u); });
    __syncthreads();
    constexpr int BPT = kNB / kSelectThreads;
    uint32_t c4[BPT];
    int sum = 0;
#pragma unroll
    for (int u = 0; u < BPT; u++) { c4[u] = cnt[tid * BPT + u]; sum += (int)c4[u]; }
    int tot;
    int base = block_exclusive_scan(sum, &tot, wsum);
#pragma unroll
    for (int u = 0; u < BPT; u++) {
        if (base < R && R <= base + (int)c4[u]) { misc[2] = tid * BPT + u; misc[3] = base + (int)c4[u]; }
        base += (int)c4[u];
    }
    if (tid == 0) misc[4] = shift;
    __syncthreads();
    return misc[3];
}

template <typename Get>
__device__ int bucket_threshold(Get get, int V, int R, const SelSmem& S)
{
    const int tid = threadIdx.x, nthr = blockDim.x;
    return bucket_threshold_each([&](auto fn) { for (int i = tid; i < V; i += nthr) fn(get(i)); }, R, S);
}

// 2b. radix threshold: exact R-th key; returns (pmask, prefix) with keep = (k & pmask) <= prefix.
template <typename Get>
__device__ void radix_threshold(Get get, int V, int R, const SelSmem& S, unsigned long long& pmask_out,
                                unsigned long long& prefix_out)
{
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5;
    unsigned long long pmask = 0ull, prefix = 0ull;
    if (V > R && R > 0) {
        // --- min / max -> highest differing bit ---
        unsigned long long mn = ~0ull, mx = 0ull;
        for (int idx = tid; idx < V; idx += nthr) { unsigned long long k = get(idx); mn = min(mn, k); mx = max(mx, k); }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mn = min(mn, __shfl_xor_sync(FULL_MASK, mn, o));
            mx = max(mx, __shfl_xor_sync(FULL_MASK, mx, o));
        }
        if (lane == 0) { S.red[warp] = mn; S.red[32 + warp] = mx; }
        __syncthreads();
        if (tid == 0) {
            unsigned long long a0 = ~0ull, a1 = 0ull;
            for (int w = 0; w < (nthr >> 5); w++) { a0 = min(a0, S.red[w]); a1 = max(a1, S.red[32 + w]); }
            S.red[0] = a0;
            S.red[32] = a1;
        }
        __syncthreads();
        mn = S.red[0];
        mx = S.red[32];
        __syncthreads();
        const int hb = 63 - __clzll((long long)(mn ^ mx));
        pmask = (hb >= 63) ? 0ull : ~((2ull << hb) - 1ull);
        prefix = mn & pmask;
        int shift = hb + 1;
        int rem = R;
        while (shift > 0) {
            const int db = shift < 8 ? shift : 8;
            shift -= db;
            const unsigned dm = (1u << db) - 1u;
            for (int t = tid; t < 16 * 256; t += nthr) S.hist[t] = 0;
            __syncthreads();
            uint32_t* hw = S.hist + (warp & 15) * 256;
            for (int idx = tid; idx < V; idx += nthr) {
                unsigned long long k = get(idx);
                if ((k & pmask) == prefix) atomicAdd(hw + ((unsigned)(k >> shift) & dm), 1u);
            }
            __syncthreads();
            for (int t = tid; t < 256; t += nthr) {
                uint32_t sum = 0;
                for (int w = 0; w < 16; w++) sum += S.hist[w * 256 + t];
                S.tot[t] = sum;
            }
            __syncthreads();
            if (warp == 0) {
                // 8 buckets per lane, lane-ordered
                uint32_t loc[8];
                uint32_t ls = 0;
#pragma unroll
                for (int u = 0; u < 8; u++) { loc[u] = S.tot[lane * 8 + u]; ls += loc[u]; }
                uint32_t inc = ls;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    uint32_t y = __shfl_up_sync(FULL_MASK, inc, o);
                    if (lane >= o) inc += y;
                }
                uint32_t before = inc - ls;
                // the bucket where the running count first reaches rem
                if ((int)before < rem && rem <= (int)inc) {
                    uint32_t cum = before;
                    for (int u = 0; u < 8; u++) {
                        if ((int)(cum + loc[u]) >= rem) {
                            S.misc[0] = lane * 8 + u;
                            S.misc[1] = (int)cum;
                            S.misc[2] = (int)loc[u];
                            break;
                        }
                        cum += loc[u];
                    }
                }
            }
            __syncthreads();
            const int dg = S.misc[0], cum = S.misc[1], cnt = S.misc[2];
            rem -= cum;
            prefix |= (unsigned long long)dg << shift;
            pmask |= (unsigned long long)dm << shift;
            __syncthreads();
            if (cnt == rem) break;
        }
    }

    pmask_out = pmask;
    prefix_out = prefix;
    __syncthreads();
}

// 3. stable compaction: each warp owns a contiguous range of the input, counted then
// written tile by tile with ballots; one block scan over the 32 warp totals.
template <typename Get, typename Keep>
__device__ int compact_stable(Get get, int V, Keep keep, unsigned long long* dst, int cap, const SelSmem& S)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    int* wtot = S.misc + 16;   // [32]
    const int L = ((V + nwarps - 1) / nwarps + 31) & ~31;
    const int lo = warp * L, hi = min(V, lo + L);
    int c = 0;
    for (int i0 = lo; i0 < hi; i0 += 32) {
        const int i = i0 + lane;
        c += __popc(__ballot_sync(FULL_MASK, i < hi && keep(get(i))));
    }
    if (lane == 0) wtot[warp] = c;
    __syncthreads();
    if (warp == 0) {
        const int v = lane < nwarps ? wtot[lane] : 0;
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL_MASK, x, o);
            if (lane >= o) x += y;
        }
        if (lane < nwarps) wtot[lane] = x - v;
        if (lane == 31) S.misc[60] = x;
    }
    __syncthreads();
    int pos = wtot[warp];
    const unsigned lt = (1u << lane) - 1u;
    for (int i0 = lo; i0 < hi; i0 += 32) {
        const int i = i0 + lane;
        unsigned long long k = 0;
        bool f = false;
        if (i < hi) { k = get(i); f = keep(k); }
        const unsigned b = __ballot_sync(FULL_MASK, f);
        if (f && pos + __popc(b & lt) < cap) dst[pos + __popc(b & lt)] = k;
        pos += __popc(b);
    }
    const int total = S.misc[60];
    __syncthreads();
    return total;
}

// 3b. dense ranks.  The survivors of a level carry few distinct scores (~150-250 at
// 50x20, K=4096: scores are cmax/ns plus a noise of a few ulps) spread over ~2^20 ulps,
// so their score bits are replaced by the rank of the score among the distinct survivor
// scores -- strictly monotone, so the (score, slot) order is unchanged -- and the radix
// sort below needs one 8-bit pass (two above 256 distinct scores) instead of three.
// Distinct scores are marked in a bitmap over the occupied buckets <= T (2^shift bits
// each); a popcount prefix over the bitmap words gives each score's rank.  Returns false,
// keys untouched, when the bitmap would not fit.  Uses the staging area above the first
// kLsdMax keys (the radix sort's second buffer) for the bitmap, its prefix and the
// occupied-bucket index.
constexpr int kDenseOccOff = kLsdMax;              // u16[kNB] occupied-bucket index
constexpr int kDenseBmOff = kLsdMax + kNB / 4;     // u32[kDenseWords] bitmap, then its prefix
constexpr int kDenseWords = 4096;
static_assert(kDenseBmOff + kDenseWords <= kStageKeys, "dense-rank tables exceed the staging area");

// Dense-rank tables over the occupied buckets <= T: a bitmap of the distinct scores
// (2^shift bits per occupied bucket) and the popcount prefix of its words.
struct DenseTables {
    uint16_t* occ;   // [kNB] occupied-bucket index
    uint32_t* bm;    // [kDenseWords] bitmap
    uint32_t* wp;    // [kDenseWords] exclusive popcount prefix of bm
    int W;           // bitmap words per occupied bucket
    int shift;
    uint32_t smin, omask;
    __device__ __forceinline__ int word_of(uint32_t score_bits, uint32_t& bit) const
    {
        const uint32_t dd = score_bits - smin;
        const uint32_t off = dd & omask;
        bit = off & 31u;
        return (int)occ[dd >> shift] * W + (int)(off >> 5);
    }
    // rank of a score among the distinct scores marked in the bitmap
    __device__ __forceinline__ uint32_t rank_of(uint32_t score_bits) const
    {
        uint32_t bit;
        const int w = word_of(score_bits, bit);
        return wp[w] + (uint32_t)__popc(bm[w] & ((1u << bit) - 1u));
    }
};

// Builds the tables for the keys `each` visits whose bucket is <= T (`each(fn)` calls fn on
// every key this thread is responsible for).  Returns the number of distinct scores, or -1
// (tables unusable) when the bitmap would exceed kDenseWords words.
template <typename ForEach>
__device__ int dense_build(ForEach each, int T, int shift, uint32_t smin, const SelSmem& S, DenseTables& D)
{
    const int tid = threadIdx.x, nthr = blockDim.x;
    D.W = shift > 5 ? 1 << (shift - 5) : 1;
    D.shift = shift;
    D.smin = smin;
    D.omask = (1u << shift) - 1u;
    int* wsum = reinterpret_cast<int*>(S.red);
    constexpr int BPT = kNB / kSelectThreads;
    int f[BPT], sum = 0;
#pragma unroll
    for (int u = 0; u < BPT; u++) {
        const int b = tid * BPT + u;
        f[u] = (b <= T && S.hist[b] != 0u) ? 1 : 0;
        sum += f[u];
    }
    int O;
    int base = block_exclusive_scan(sum, &O, wsum);
#pragma unroll
    for (int u = 0; u < BPT; u++) {
        D.occ[tid * BPT + u] = (uint16_t)base;
        base += f[u];
    }
    const int nw = O * D.W;
    if (nw > kDenseWords) return -1;   // O is the same in every thread
    for (int w = tid; w < nw; w += nthr) D.bm[w] = 0u;
    __syncthreads();
    const uint32_t lim = ((uint32_t)T + 1u) << shift;
    each([&](unsigned long long k) {
        const uint32_t sb = (uint32_t)(k >> 32);
        if (sb - smin < lim) {
            uint32_t bit;
            const int w = D.word_of(sb, bit);
            atomicOr(&D.bm[w], 1u << bit);
        }
    });
    __syncthreads();
    const int per = (nw + nthr - 1) / nthr;
    int c = 0;
    for (int k = 0; k < per; k++) {
        const int w = tid * per + k;
        if (w < nw) c += __popc(D.bm[w]);
    }
    int Dn;
    int pre = block_exclusive_scan(c, &Dn, wsum);
    for (int k = 0; k < per; k++) {
        const int w = tid * per + k;
        if (w < nw) {
            D.wp[w] = (uint32_t)pre;
            pre += __popc(D.bm[w]);
        }
    }
    __syncthreads();
    return Dn;
}

// 4'. One stable counting pass over the compacted survivors by their dense score rank (at
// most 256 distinct), scattered straight into `sel`.  The rank of each element comes from
// the dense tables as it is loaded: no min/max pass, no second buffer, no emit pass.
// Elements p = warp*32*E + e*32 + lane (warps own contiguous runs, E = ceil(count/1024))
// are ranked in element order against per-warp 16-bit digit counters with bit-ballot peer
// masks; each element's (rank, offset) goes back into its own A slot (bits 63..48 rank,
// 47..32 offset) so the loops stay rolled; a digit-major prefix over (digit, warp) gives
// the positions.
__device__ void dense_sort_emit(unsigned long long* A, int count, int R, const DenseTables& D, uint32_t* sel,
                                       const SelSmem& S)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const int E = (count + kSelectThreads - 1) / kSelectThreads;
    uint16_t* wh = reinterpret_cast<uint16_t*>(S.hist);   // [32][256]
    int* dtot = reinterpret_cast<int*>(S.tot);           // [256]
    for (int i = tid; i < 32 * 256 / 2; i += blockDim.x) S.hist[i] = 0u;
    __syncthreads();
#pragma unroll 1
    for (int e = 0; e < E; e++) {
        const int p = warp * 32 * E + e * 32 + lane;
        const bool valid = p < count;
        const unsigned long long x = valid ? A[p] : 0ull;
        const int d = valid ? (int)D.rank_of((uint32_t)(x >> 32)) : 0;
        unsigned grp = __ballot_sync(FULL_MASK, valid);
#pragma unroll
        for (int bit = 0; bit < 8; bit++) {
            const unsigned bb = __ballot_sync(FULL_MASK, (d >> bit) & 1);
            grp &= ((d >> bit) & 1) ? bb : ~bb;
        }
        const int r_in = __popc(grp & lt);
        int b = 0;
        if (valid) b = wh[warp * 256 + d];
        __syncwarp();
        if (valid && r_in == 0) wh[warp * 256 + d] = (uint16_t)(b + __popc(grp));
        __syncwarp();
        if (valid)
            A[p] = ((unsigned long long)d << 48) | ((unsigned long long)(b + r_in) << 32) | (x & 0xFFFFFFFFull);
    }
    __syncthreads();
    if (tid < 256) {
        int run = 0;
        for (int w = 0; w < 32; w++) {
            const int t = wh[w * 256 + tid];
            wh[w * 256 + tid] = (uint16_t)run;
            run += t;
        }
        dtot[tid] = run;
    }
    __syncthreads();
    if (warp == 0) {
        int v8[8], sum = 0;
#pragma unroll
        for (int u = 0; u < 8; u++) { v8[u] = dtot[lane * 8 + u]; sum += v8[u]; }
        int xx = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL_MASK, xx, o);
            if (lane >= o) xx += y;
        }
        int run = xx - sum;
#pragma unroll
        for (int u = 0; u < 8; u++) { dtot[lane * 8 + u] = run; run += v8[u]; }
    }
    __syncthreads();
#pragma unroll 1
    for (int e = 0; e < E; e++) {
        const int p = warp * 32 * E + e * 32 + lane;
        if (p < count) {
            const unsigned long long x = A[p];
            const int dg = (int)(x >> 48);
            const int pos = dtot[dg] + (int)wh[warp * 256 + dg] + (int)((x >> 32) & 0xFFFFull);
            if (pos < R) sel[pos] = (uint32_t)(x & 0xFFFFFFFFull);
        }
    }
}

// 4. stable LSD radix sort of `count` (<= kLsdMax) keys by their score bits, first R out.
// Elements p = warp*32*E + e*32 + lane are ranked in element order against per-warp
// 16-bit digit counters with bit-ballot peer masks (no atomics); a digit-major prefix over
// (digit, warp) gives the scatter base.
template <int E>
__device__ unsigned long long* lsd_sort(unsigned long long* A, unsigned long long* B, int count, const SelSmem& S)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt = (1u << lane) - 1u;
    uint16_t* wh = reinterpret_cast<uint16_t*>(S.hist);   // [32][256]
    int* dtot = reinterpret_cast<int*>(S.tot);
    int* misc = S.misc;
    uint32_t mn = 0xFFFFFFFFu, mx = 0u;
#pragma unroll
    for (int e = 0; e < E; e++) {
        const int p = warp * 32 * E + e * 32 + lane;
        if (p < count) { const uint32_t sb = (uint32_t)(A[p] >> 32); mn = min(mn, sb); mx = max(mx, sb); }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = min(mn, __shfl_xor_sync(FULL_MASK, mn, o));
        mx = max(mx, __shfl_xor_sync(FULL_MASK, mx, o));
    }
    if (tid == 0) { misc[8] = 0; misc[9] = (int)0xFFFFFFFFu; }
    __syncthreads();
    if (lane == 0) {
        atomicMax(reinterpret_cast<unsigned*>(&misc[8]), mx);
        atomicMin(reinterpret_cast<unsigned*>(&misc[9]), mn);
    }
    __syncthreads();
    const uint32_t smin = (uint32_t)misc[9];
    const uint32_t range = (uint32_t)misc[8] - smin;
    const int nbits = (count > 0 && range) ? 32 - __clz(range) : 0;
    for (int sh = 0; sh < nbits; sh += 8) {
        uint32_t* wh32 = S.hist;
        for (int i = tid; i < 32 * 256 / 2; i += blockDim.x) wh32[i] = 0;
        __syncthreads();
        unsigned long long x[E];
        int dg[E], off[E];
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int p = warp * 32 * E + e * 32 + lane;
            const bool valid = p < count;
            x[e] = valid ? A[p] : 0ull;
            const int d = valid ? (int)(((((uint32_t)(x[e] >> 32)) - smin) >> sh) & 255u) : 0;
            // lanes holding the same digit: intersect the 8 bit-ballots
            unsigned grp = __ballot_sync(FULL_MASK, valid);
#pragma unroll
            for (int bit = 0; bit < 8; bit++) {
                const unsigned bb = __ballot_sync(FULL_MASK, (d >> bit) & 1);
                grp &= ((d >> bit) & 1) ? bb : ~bb;
            }
            const int r_in = __popc(grp & lt);
            int b = 0;
            if (valid) b = wh[warp * 256 + d];
            __syncwarp();
            if (valid && r_in == 0) wh[warp * 256 + d] = (uint16_t)(b + __popc(grp));
            __syncwarp();
            dg[e] = d;
            off[e] = b + r_in;
        }
        __syncthreads();
        // per digit: exclusive prefix over the 32 warps (thread d walks the warps; the
        // [warp][256] layout makes consecutive threads read consecutive counters)
        if (tid < 256) {
            int run = 0;
            for (int w = 0; w < 32; w++) {
                const int t = wh[w * 256 + tid];
                wh[w * 256 + tid] = (uint16_t)run;
                run += t;
            }
            dtot[tid] = run;
        }
        __syncthreads();
        if (warp == 0) {
            int v8[8], sum = 0;
#pragma unroll
            for (int u = 0; u < 8; u++) { v8[u] = dtot[lane * 8 + u]; sum += v8[u]; }
            int xx = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(FULL_MASK, xx, o);
                if (lane >= o) xx += y;
            }
            int run = xx - sum;
#pragma unroll
            for (int u = 0; u < 8; u++) { dtot[lane * 8 + u] = run; run += v8[u]; }
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int p = warp * 32 * E + e * 32 + lane;
            if (p < count) B[dtot[dg[e]] + (int)wh[warp * 256 + dg[e]] + off[e]] = x[e];
        }
        __syncthreads();
        unsigned long long* t = A;
        A = B;
        B = t;
    }
    return A;
}

template <int E>
__device__ void lsd_sort_emit(unsigned long long* A, unsigned long long* B, int count, int R, uint32_t* sel,
                              const SelSmem& S)
{
    const unsigned long long* out = lsd_sort<E>(A, B, count, S);
    for (int i = threadIdx.x; i < R; i += blockDim.x) sel[i] = (uint32_t)(out[i] & 0xFFFFFFFFull);
}

// in-thread compare-exchange stage of distance J (< E) on the blocked layout i = t*E + e
template <int E, int J>
__device__ __forceinline__ void bitonic_in_thread(unsigned long long (&x)[E], int t, int k)
{
#pragma unroll
    for (int e = 0; e < E; e++) {
        if ((e & J) == 0) {
            const bool up = ((t * E + e) & k) == 0;
            const unsigned long long a = x[e], b = x[e + J];
            if ((a > b) == up) { x[e] = b; x[e + J] = a; }
        }
    }
}

// Ascending bitonic sort of N = 1024*E keys, E per thread (thread t holds positions
// t*E .. t*E+E-1); xs is a shared exchange buffer of N keys, used striped (e*1024 + t) so
// cross-warp stages are bank-conflict free.
template <int E>
__device__ void block_bitonic_reg(unsigned long long (&x)[E], unsigned long long* xs)
{
    const int t = threadIdx.x, lane = t & 31;
    const int N = E * kSelectThreads;
    for (int k = 2; k <= N; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j < E) {
                if (j == 1) bitonic_in_thread<E, 1>(x, t, k);
                else if (j == 2) bitonic_in_thread<E, (E > 2 ? 2 : 1)>(x, t, k);
                else if (j == 4) bitonic_in_thread<E, (E > 4 ? 4 : 1)>(x, t, k);
                else bitonic_in_thread<E, (E > 8 ? 8 : 1)>(x, t, k);
            } else if (j < 32 * E) {
                const int lj = j / E;
                const bool low = (lane & lj) == 0;
#pragma unroll
                for (int e = 0; e < E; e++) {
                    const bool up = ((t * E + e) & k) == 0;
                    const unsigned long long y = __shfl_xor_sync(FULL_MASK, x[e], lj);
                    x[e] = (low == up) ? umin64(x[e], y) : umax64(x[e], y);
                }
            } else {
                const int tj = j / E;
#pragma unroll
                for (int e = 0; e < E; e++) xs[e * kSelectThreads + t] = x[e];
                __syncthreads();
                const bool low = (t & tj) == 0;
#pragma unroll
                for (int e = 0; e < E; e++) {
                    const bool up = ((t * E + e) & k) == 0;
                    const unsigned long long y = xs[e * kSelectThreads + (t ^ tj)];
                    x[e] = (low == up) ? umin64(x[e], y) : umax64(x[e], y);
                }
                __syncthreads();
            }
        }
    }
}

template <int E>
__device__ void sort_emit_e(unsigned long long* sbuf, int count, int R, uint32_t* sel)
{
    const int t = threadIdx.x;
    unsigned long long x[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
        const int idx = e * kSelectThreads + t;   // any bijection works for unsorted input
        x[e] = idx < count ? sbuf[idx] : ~0ull;
    }
    __syncthreads();
    block_bitonic_reg<E>(x, sbuf);
#pragma unroll
    for (int e = 0; e < E; e++) {
        const int i = t * E + e;
        if (i < R) sel[i] = (uint32_t)(x[e] & 0xFFFFFFFFull);
    }
}

// Sort the `count` keys in sbuf and write the first R slots to sel (count <= 16384).
__device__ void sort_and_emit(unsigned long long* sbuf, int count, int R, uint32_t* sel)
{
    const int N = pow2ceil(count);
    if (N <= kSelectThreads) sort_emit_e<1>(sbuf, count, R, sel);
    else if (N <= 2 * kSelectThreads) sort_emit_e<2>(sbuf, count, R, sel);
    else if (N <= 4 * kSelectThreads) sort_emit_e<4>(sbuf, count, R, sel);
    else if (N <= 8 * kSelectThreads) sort_emit_e<8>(sbuf, count, R, sel);
    else sort_emit_e<16>(sbuf, count, R, sel);
}

// Fillers (v1 / v2 only): when fewer than min(P*n, K) children were scored, the
// reference's stable sort keeps the lowest-numbered unscored slots next, in slot order.
__device__ void select_fillers(const SegDesc& d, const StepArgs& a, int P, int R, int keff, uint32_t* sel,
                               uint8_t* smem)
{
    if (keff <= R) return;
    int* wsum = reinterpret_cast<int*>(smem);
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int n = d.n;
    const int F = keff - R;
    const int W = d.words;
    const uint32_t* mk = a.masks + d.mask_off;
    int base = 0;
    for (int c0 = 0; c0 < P && base < F; c0 += nthr) {
        const int c = c0 + tid;
        int f = 0;
        if (c < P) {
            int pc = 0;
            for (int w = 0; w < W; w++) pc += __popc(mk[(int64_t)c * W + w]);
            f = n - pc;
        }
        int tot;
        const int off = block_exclusive_scan(f, &tot, wsum);
        if (c < P && base + off < F) {
            int out = R + base + off;
            const int lim = F - base - off;
            int got = 0;
            for (int b = 0; b < n && got < lim && got < f; b++) {
                uint32_t word = mk[(int64_t)c * W + (b >> 5)];
                if (!((word >> (b & 31)) & 1u)) {
                    sel[out + got] = kFillerFlag | (uint32_t)(c * n + b);
                    got++;
                }
            }
        }
        base += tot;
    }
}

// ---- large levels: more candidate keys than the staging area holds (V > kStageKeys) or
// more survivors than the 64-bit radix buffer (K > kLsdMax).  The keys stay in their chunk
// regions in global memory (L2-resident); survivors are compacted as 32-bit words
// (dense rank << 21 | slot) into the two 96 KB halves of the A/stg area, and sorted by the
// rank bits with a stable 8-bit radix pass that needs no per-element registers. ----
constexpr int kBigCap = kLsdMax + kStageKeys;  // u32 survivors per half of the A/stg area
constexpr int kSlotBits = 21;                                         // slot < K * n <= 2^21
constexpr int kBigMaxDistinct = 1 << (32 - kSlotBits);                // ranks in the top 11 bits
static_assert(2 * kBigCap * 4 == (kLsdMax + kStageKeys) * 8, "two kBigCap u32 halves fill the A/stg area");
static_assert(kNB / 2 + 2 * kDenseWords <= kBigCap, "dense tables must fit the second half");
static_assert((long long)kMaxBeam * kMaxJobs <= (1LL << kSlotBits), "slots must fit 21 bits");

// Stable compaction of the keys of buckets <= T (score bits - smin < lim), in slot order,
// each written as (dense rank << kSlotBits) | slot.  Warps own contiguous runs of chunks:
// one counting sweep, a scan of the warp totals, one writing sweep.
__device__ int compact_ranked(const KeySrc& ks, uint32_t lim, uint32_t smin, const DenseTables& D, uint32_t* out,
                              int cap, const SelSmem& S)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    int* wtot = S.misc + 16;   // [32]
    const int cpw = (ks.nch + nwarps - 1) / nwarps;
    const int c_lo = min(ks.nch, warp * cpw), c_hi = min(ks.nch, c_lo + cpw);
    int c = 0;
    for (int ch = c_lo; ch < c_hi; ch++) {
        const int nc = ks.cpref[ch + 1] - ks.cpref[ch];
        const unsigned long long* src = ks.base + (size_t)ch * ks.cap;
        for (int j0 = 0; j0 < nc; j0 += 32) {
            const int j = j0 + lane;
            const bool f = j < nc && ((uint32_t)(src[j] >> 32) - smin) < lim;
            c += __popc(__ballot_sync(FULL_MASK, f));
        }
    }
    if (lane == 0) wtot[warp] = c;
    __syncthreads();
    if (warp == 0) {
        const int v = lane < nwarps ? wtot[lane] : 0;
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL_MASK, x, o);
            if (lane >= o) x += y;
        }
        if (lane < nwarps) wtot[lane] = x - v;
        if (lane == 31) S.misc[60] = x;
    }
    __syncthreads();
    int pos = wtot[warp];
    const unsigned lt = (1u << lane) - 1u;
    for (int ch = c_lo; ch < c_hi; ch++) {
        const int nc = ks.cpref[ch + 1] - ks.cpref[ch];
        const unsigned long long* src = ks.base + (size_t)ch * ks.cap;
        for (int j0 = 0; j0 < nc; j0 += 32) {
            const int j = j0 + lane;
            unsigned long long k = 0;
            bool f = false;
            if (j < nc) {
                k = src[j];
                f = ((uint32_t)(k >> 32) - smin) < lim;
            }
            const unsigned b = __ballot_sync(FULL_MASK, f);
            const int at = pos + __popc(b & lt);
            if (f && at < cap) out[at] = (D.rank_of((uint32_t)(k >> 32)) << kSlotBits) | (uint32_t)(k & 0xFFFFFFFFull);
            pos += __popc(b);
        }
    }
    const int total = S.misc[60];
    __syncthreads();
    return total;
}

// One stable counting pass of src[0..count) into dst by the 8-bit digit at bit `sh`.
// Warps own contiguous element runs; a digit's rank inside a 32-element tile comes from the
// peers' bit ballots, across tiles and warps from per-warp 16-bit counters.  The tiles are
// walked twice (count, then scatter) so no element state is held across the prefix.
__device__ void radix_pass32(const uint32_t* src, uint32_t* dst, int count, int sh, const SelSmem& S)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    uint16_t* wh = reinterpret_cast<uint16_t*>(S.hist);   // [32][256]
    int* dtot = reinterpret_cast<int*>(S.tot);           // [256]
    const unsigned lt = (1u << lane) - 1u;
    const int per = ((count + nwarps - 1) / nwarps + 31) & ~31;
    const int lo = min(count, warp * per), hi = min(count, lo + per);
    for (int i = tid; i < 32 * 256 / 2; i += blockDim.x) S.hist[i] = 0u;
    __syncthreads();
    auto peers = [&](bool valid, int dg) {
        unsigned grp = __ballot_sync(FULL_MASK, valid);
#pragma unroll
        for (int bit = 0; bit < 8; bit++) {
            const unsigned bb = __ballot_sync(FULL_MASK, (dg >> bit) & 1);
            grp &= ((dg >> bit) & 1) ? bb : ~bb;
        }
        return grp;
    };
    for (int i0 = lo; i0 < hi; i0 += 32) {
        const int i = i0 + lane;
        const bool valid = i < hi;
        const int dg = valid ? (int)((src[i] >> sh) & 255u) : 0;
        const unsigned grp = peers(valid, dg);
        if (valid && (grp & lt) == 0u) wh[warp * 256 + dg] = (uint16_t)(wh[warp * 256 + dg] + __popc(grp));
        __syncwarp();
    }
    __syncthreads();
    if (tid < 256) {
        int run = 0;
        for (int w = 0; w < nwarps; w++) {
            const int t = wh[w * 256 + tid];
            wh[w * 256 + tid] = (uint16_t)run;
            run += t;
        }
        dtot[tid] = run;
    }
    __syncthreads();
    if (warp == 0) {
        int v8[8], sum = 0;
#pragma unroll
        for (int u = 0; u < 8; u++) { v8[u] = dtot[lane * 8 + u]; sum += v8[u]; }
        int xx = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL_MASK, xx, o);
            if (lane >= o) xx += y;
        }
        int run = xx - sum;
#pragma unroll
        for (int u = 0; u < 8; u++) { dtot[lane * 8 + u] = run; run += v8[u]; }
    }
    __syncthreads();
    for (int i0 = lo; i0 < hi; i0 += 32) {
        const int i = i0 + lane;
        const bool valid = i < hi;
        const uint32_t x = valid ? src[i] : 0u;
        const int dg = (int)((x >> sh) & 255u);
        const unsigned grp = peers(valid, dg);
        if (valid) dst[dtot[dg] + (int)wh[warp * 256 + dg] + __popc(grp & lt)] = x;
        __syncwarp();
        if (valid && (grp & lt) == 0u) wh[warp * 256 + dg] = (uint16_t)(wh[warp * 256 + dg] + __popc(grp));
        __syncwarp();
    }
    __syncthreads();
}

// The whole selection of a large level; false (nothing written) when it does not fit
// these buffers -- then the general path runs.
__device__ bool select_large(SegState& st, int R, const KeySrc& ks, uint32_t* sel, const SelSmem& S)
{
    const int tid = threadIdx.x;
    auto each = [&](auto fn) { ks.each_key(fn); };
    const int count0 = bucket_threshold_each(each, R, S);
    const int T = S.misc[2], shift = S.misc[4];
    const uint32_t smin = (uint32_t)S.misc[1];
    __syncthreads();
    if (count0 > kBigCap) return false;
    uint32_t* buf1 = reinterpret_cast<uint32_t*>(S.A);
    uint32_t* buf2 = buf1 + kBigCap;
    DenseTables D;
    D.occ = reinterpret_cast<uint16_t*>(buf2);
    D.bm = buf2 + kNB / 2;
    D.wp = D.bm + kDenseWords;
    const int nd = dense_build(each, T, shift, smin, S, D);
    if (nd < 0 || nd > kBigMaxDistinct) return false;
    const uint32_t lim = ((uint32_t)T + 1u) << shift;
    int count = compact_ranked(ks, lim, smin, D, buf1, kBigCap, S);
    if (count != count0 || count < R) {
        if (tid == 0) atomicOr(&st.status, kStatusBadSelect);
        count = min(count, kBigCap);
    }
    const int nbits = nd > 1 ? 32 - __clz(nd - 1) : 0;
    uint32_t* src = buf1;
    uint32_t* dst = buf2;
    for (int sh = kSlotBits; sh < kSlotBits + nbits; sh += 8) {
        radix_pass32(src, dst, count, sh, S);
        uint32_t* t = src;
        src = dst;
        dst = t;
    }
    const int RR = R < count ? R : count;
    for (int i = tid; i < RR; i += blockDim.x) sel[i] = src[i] & ((1u << kSlotBits) - 1u);
    __syncthreads();
    return true;
}

// ---- direct staged selection: the common case of a level that fits the staging area.
// After the bucket threshold, the distinct scores of the keys of buckets <= T get dense
// ranks (at most 256 of them); one stable counting pass over the staged keys, in slot
// order, then gives every kept key its final position in (score, slot) order -- the
// reference's stable sort order -- and survivors below R go straight to `sel`.  Warps own
// contiguous runs of the staged keys: pass 1 walks each run tile by tile, ranking a key
// against its tile peers (bit ballots of the digit) and the warp's running per-digit
// counters, and writes (digit << 16 | offset) over the key's score bits; after a
// digit-major prefix over (digit, warp), pass 2 scatters in parallel.  No compaction
// buffer, no sort passes.  Returns false -- staged keys untouched, nothing written -- when
// the dense tables do not fit or there are more than 256 distinct scores; the general
// path then runs.  Taken for levels of up to kDirectMaxKeys keys. ----
constexpr int kDirectMaxDistinct = 256;
// Largest level (candidate keys) the direct path takes: beyond it, compacting the keys
// first and sorting the survivors is faster (a GB300 sweep over 18 shapes: the direct
// path wins 5-10 % up to ~4 K keys, loses from ~6 K on).
constexpr int kDirectMaxKeys = 4096;

__device__ bool select_direct(unsigned long long* stg, int V, int R, int T, int shift, uint32_t smin, uint32_t* sel,
                              const SelSmem& S)
{
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;
    DenseTables D;
    D.occ = reinterpret_cast<uint16_t*>(S.A);
    D.bm = reinterpret_cast<uint32_t*>(S.A + kNB / 4);
    D.wp = D.bm + kDenseWords;
    auto each = [&](auto fn) {
        for (int i = tid; i < V; i += nthr) fn(stg[i]);
    };
    const int nd = dense_build(each, T, shift, smin, S, D);   // reads S.hist, ends synchronised
    if (nd < 0 || nd > kDirectMaxDistinct) return false;      // the same in every thread
    uint16_t* wh = reinterpret_cast<uint16_t*>(S.hist);       // [32][256] per-warp digit counters
    int* dtot = reinterpret_cast<int*>(S.tot);                // [256]
    for (int i = tid; i < 32 * 256 / 2; i += nthr) S.hist[i] = 0u;
    __syncthreads();
    const uint32_t lim = ((uint32_t)T + 1u) << shift;          // bucket <= T
    const unsigned lt = (1u << lane) - 1u;
    const int per = ((V + nwarps - 1) / nwarps + 31) & ~31;   // <= 512: offsets fit 16 bits
    const int lo = min(V, warp * per), hi = min(V, lo + per);
    // two tiles per step: their digits and peer sets are independent; only the counter
    // updates run in tile order
    auto tile = [&](int i, unsigned long long& k, int& dg, unsigned& grp) {
        k = ~0ull;
        dg = 0;
        bool kept = false;
        if (i < hi) {
            k = stg[i];
            const uint32_t sb = (uint32_t)(k >> 32);
            kept = (sb - smin) < lim;
            if (kept) dg = (int)D.rank_of(sb);
        }
        grp = __ballot_sync(FULL_MASK, kept);
#pragma unroll
        for (int bit = 0; bit < 8; bit++) {
            const unsigned bb = __ballot_sync(FULL_MASK, (dg >> bit) & 1);
            grp &= ((dg >> bit) & 1) ? bb : ~bb;
        }
        if (!kept) grp = 0u;
    };
    auto count = [&](int dg, unsigned grp) {
        int base = 0;
        if (grp) base = wh[warp * 256 + dg];
        __syncwarp();
        if (grp && (grp & lt) == 0u) wh[warp * 256 + dg] = (uint16_t)(base + __popc(grp));
        __syncwarp();
        return base + __popc(grp & lt);
    };
    for (int i0 = lo; i0 < hi; i0 += 64) {
        const int ia = i0 + lane, ib = i0 + 32 + lane;
        unsigned long long ka, kb;
        int da, db;
        unsigned ga, gb;
        tile(ia, ka, da, ga);
        tile(ib, kb, db, gb);
        const int oa = count(da, ga);
        const int ob = count(db, gb);
        if (ia < hi) stg[ia] = ga ? ((unsigned long long)(((uint32_t)da << 16) | (uint32_t)oa) << 32) | (ka & 0xFFFFFFFFull) : ~0ull;
        if (ib < hi) stg[ib] = gb ? ((unsigned long long)(((uint32_t)db << 16) | (uint32_t)ob) << 32) | (kb & 0xFFFFFFFFull) : ~0ull;
    }
    __syncthreads();
    // per digit: exclusive prefix over the warps, then over the digits
    if (tid < 256) {
        int run = 0;
        for (int w = 0; w < nwarps; w++) {
            const int t = wh[w * 256 + tid];
            wh[w * 256 + tid] = (uint16_t)run;
            run += t;
        }
        dtot[tid] = run;
    }
    __syncthreads();
    if (warp == 0) {
        int v8[8], sum = 0;
#pragma unroll
        for (int u = 0; u < 8; u++) { v8[u] = dtot[lane * 8 + u]; sum += v8[u]; }
        int xx = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL_MASK, xx, o);
            if (lane >= o) xx += y;
        }
        int run = xx - sum;
#pragma unroll
        for (int u = 0; u < 8; u++) { dtot[lane * 8 + u] = run; run += v8[u]; }
    }
    __syncthreads();
    for (int i = tid; i < V; i += nthr) {
        const unsigned long long x = stg[i];
        const uint32_t h = (uint32_t)(x >> 32);
        if (h != 0xFFFFFFFFu) {
            const int dg = (int)(h >> 16);
            const int pos = dtot[dg] + (int)wh[(i / per) * 256 + dg] + (int)(h & 0xFFFFu);
            if (pos < R) sel[pos] = (uint32_t)(x & 0xFFFFFFFFull);
        }
    }
    __syncthreads();
    return true;
}

// lsd_sort_emit for any count <= kLsdMax (E = ceil(count / kSelectThreads) elements per thread)
__device__ void lsd_sort_emit_n(unsigned long long* A, unsigned long long* B, int count, int R, uint32_t* sel,
                                const SelSmem& S)
{
    switch ((count + kSelectThreads - 1) / kSelectThreads) {
    case 0:
    case 1: lsd_sort_emit<1>(A, B, count, R, sel, S); break;
    case 2: lsd_sort_emit<2>(A, B, count, R, sel, S); break;
    case 3: lsd_sort_emit<3>(A, B, count, R, sel, S); break;
    case 4: lsd_sort_emit<4>(A, B, count, R, sel, S); break;
    case 5: lsd_sort_emit<5>(A, B, count, R, sel, S); break;
    case 6: lsd_sort_emit<6>(A, B, count, R, sel, S); break;
    case 7: lsd_sort_emit<7>(A, B, count, R, sel, S); break;
    default: lsd_sort_emit<8>(A, B, count, R, sel, S); break;
    }
}

__device__ void select_gpu(const SegDesc& d, SegState& st, const StepArgs& a, int P, int V, const KeySrc& ks,
                           uint8_t* smem, uint32_t rmin, uint32_t rmax)
{
    const int tid = threadIdx.x;
    const int K = d.K;
    const int total = P * d.n;
    const int keff = (d.mode == MODE_CLEAN) ? (V < K ? V : K) : (total < K ? total : K);
    const int R = V < keff ? V : keff;
    uint32_t* sel = a.sel + d.sel_off;
    const SelSmem S = sel_smem(smem, rmin, rmax);
    const int fz = a.select_force;    // route flags (0 = by level size); uniform over the block
    // routes taken, recorded by thread 0 with a reduction that returns nothing
    auto route = [&](uint32_t bit) { if (tid == 0) atomicOr(&st.select_paths, bit); };
    // staged (shared-memory) input when the level fits; larger levels take select_large
    const bool staged = (V <= kStageKeys) && (K <= kLsdMax);
    const bool try_large = (fz & kSelForceLarge) ? true : ((fz & kSelNoLarge) ? false : !staged);
    if (R > 0 && try_large && select_large(st, R, ks, sel, S)) {
        route(kPathLarge);   // done: survivors 0..R-1 written
    } else if (R > 0) {
        if (staged) stage_keys(ks, S.stg);
        const unsigned long long* stg = S.stg;
        auto get_s = [=](int i) { return stg[i]; };
        auto get_g = [=](int i) { return ks(i); };
        int count = staged ? bucket_threshold(get_s, V, R, S) : bucket_threshold(get_g, V, R, S);
        unsigned long long* dst = S.A;
        const int T = S.misc[2], shift = S.misc[4];
        const uint32_t smin = (uint32_t)S.misc[1];
        // survivors = the keys of buckets <= T
        const bool bucketed = count <= kLsdMax && !(fz & kSelForceRadix);
        __syncthreads();
        const bool direct = !(fz & (kSelNoDirect | kSelForceRadix)) && staged && V <= kDirectMaxKeys &&
                            count >= R && select_direct(S.stg, V, R, T, shift, smin, sel, S);
        if (direct) route(kPathDirect);
        if (!direct) {
            if (bucketed) {
                route(kPathBucket);
                const uint32_t lim = ((uint32_t)T + 1u) << shift;  // bucket <= T
                auto keep = [=](unsigned long long k) { return (((uint32_t)(k >> 32)) - smin) < lim; };
                count = staged ? compact_stable(get_s, V, keep, dst, kLsdMax, S)
                               : compact_stable(get_g, V, keep, dst, kLsdMax, S);
            } else {
                route(kPathRadix);
                if (tid == 0) st.select_fallbacks += 1;
                unsigned long long pmask, prefix;
                if (staged) radix_threshold(get_s, V, R, S, pmask, prefix);
                else radix_threshold(get_g, V, R, S, pmask, prefix);
                auto keep = [=](unsigned long long k) { return (k & pmask) <= prefix; };
                if (R > kLsdMax) dst = S.stg;  // only reached unstaged (K > kLsdMax)
                const int cap = (R > kLsdMax) ? kStageKeys : kLsdMax;
                count = staged ? compact_stable(get_s, V, keep, dst, cap, S)
                               : compact_stable(get_g, V, keep, dst, cap, S);
            }
            if (count < R || count > kStageKeys) {
                if (tid == 0) atomicOr(&st.status, kStatusBadSelect);
                count = count > kStageKeys ? kStageKeys : count;
            }
            const int RR = R < count ? R : count;
            if (count <= kLsdMax && !(fz & kSelBitonic)) {
                int nd = -1;
                DenseTables D;
                if (bucketed && !(fz & kSelNoDense)) {
                    // bucket counts are intact on the bucketed path (the radix path reuses them)
                    D.occ = reinterpret_cast<uint16_t*>(S.stg + kDenseOccOff);
                    D.bm = reinterpret_cast<uint32_t*>(S.stg + kDenseBmOff);
                    D.wp = D.bm + kDenseWords;
                    auto each = [&](auto fn) {
                        for (int i = tid; i < count; i += kSelectThreads) fn(dst[i]);
                    };
                    nd = dense_build(each, T, shift, smin, S, D);
                }
                if (nd >= 0 && nd <= 256 && !(fz & kSelRankLsd)) {
                    route(kPathDense);
                    dense_sort_emit(dst, count, RR, D, sel, S);
                } else {
                    if (nd >= 0) {
                        // more distinct scores than one 8-bit pass (or the route is forced):
                        // ranks into the keys, then LSD passes over the rank bits
                        route(kPathRankLsd);
                        for (int i = tid; i < count; i += kSelectThreads) {
                            const unsigned long long k = dst[i];
                            dst[i] = ((unsigned long long)D.rank_of((uint32_t)(k >> 32)) << 32) | (k & 0xFFFFFFFFull);
                        }
                        __syncthreads();
                    } else {
                        route(kPathRawLsd);
                    }
                    lsd_sort_emit_n(dst, S.stg, count, RR, sel, S);
                }
            } else {
                route(kPathBitonic);
                if (dst != S.stg) {
                    // survivors in A (count <= kLsdMax): the bitonic sort works in stg
                    for (int i = tid; i < count; i += kSelectThreads) S.stg[i] = dst[i];
                    __syncthreads();
                }
                sort_and_emit(S.stg, count, RR, sel);
            }
        }
    }
    __syncthreads();
    select_fillers(d, a, P, R, keff, sel, smem);
    __syncthreads();
    if (tid == 0) {
        st.P = keff;
        atomicAdd(reinterpret_cast<unsigned long long*>(&st.materialized), (unsigned long long)keff);
    }
}

// Candidate counts of the level's chunks -> their prefix in s_cpref (nch + 1 entries, up to
// 2 chunks per thread); returns V, the level's candidate keys, and in rmin / rmax the min
// and max score bits over the chunks' ranges.  One block scan carries the sum and both
// reductions; s_red: 100 words of scratch.  Ends synchronised.
__device__ int level_key_prefix(const StepArgs& a, const SegDesc& d, int nch, int* s_cpref, uint32_t* s_red,
                                uint32_t& rmin, uint32_t& rmax)
{
    constexpr int CPT = (kMaxChunks + kSelectThreads - 1) / kSelectThreads;
    const int c0 = threadIdx.x * CPT, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    uint32_t* wsum = s_red;        // [32] warp sums, then their exclusive prefixes
    uint32_t* wmin = s_red + 32;   // [32]
    uint32_t* wmax = s_red + 64;   // [32]
    uint32_t* res = s_red + 96;    // [3] total, min, max
    int cv[CPT], v = 0;
    uint32_t mn = 0xFFFFFFFFu, mx = 0u;
#pragma unroll
    for (int u = 0; u < CPT; u++) {
        cv[u] = 0;
        if (c0 + u < nch) {
            cv[u] = a.kcnt[d.kcnt_off + c0 + u];
            const uint2 r = a.kmm[d.kcnt_off + c0 + u];
            mn = min(mn, r.x);
            mx = max(mx, r.y);
        }
        v += cv[u];
    }
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL_MASK, x, o);
        if (lane >= o) x += y;
        mn = min(mn, __shfl_xor_sync(FULL_MASK, mn, o));
        mx = max(mx, __shfl_xor_sync(FULL_MASK, mx, o));
    }
    if (lane == 31) wsum[warp] = (uint32_t)x;
    if (lane == 0) { wmin[warp] = mn; wmax[warp] = mx; }
    __syncthreads();
    if (warp == 0) {
        const int w = lane < nwarps ? (int)wsum[lane] : 0;
        uint32_t m0 = lane < nwarps ? wmin[lane] : 0xFFFFFFFFu, m1 = lane < nwarps ? wmax[lane] : 0u;
        int ws = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL_MASK, ws, o);
            if (lane >= o) ws += y;
            m0 = min(m0, __shfl_xor_sync(FULL_MASK, m0, o));
            m1 = max(m1, __shfl_xor_sync(FULL_MASK, m1, o));
        }
        wsum[lane] = (uint32_t)(ws - w);
        if (lane == 31) { res[0] = (uint32_t)ws; res[1] = m0; res[2] = m1; }
    }
    __syncthreads();
    int pre = (int)wsum[warp] + x - v;
    const int V = (int)res[0];
    rmin = res[1];
    rmax = res[2];
#pragma unroll
    for (int u = 0; u < CPT; u++) {
        if (c0 + u < nch) s_cpref[c0 + u] = pre;
        pre += cv[u];
    }
    if (threadIdx.x == 0) s_cpref[nch] = V;
    __syncthreads();
    return V;
}

// The level's counters, as reductions (no round trip on the selection's path).
__device__ __forceinline__ void count_level(int n, SegState& st, int P, int V)
{
    atomicAdd(reinterpret_cast<unsigned long long*>(&st.expanded), (unsigned long long)V);
    atomicAdd(reinterpret_cast<unsigned long long*>(&st.slots), (unsigned long long)P * (unsigned long long)n);
    if (P > 0) atomicAdd(&st.levels, 1);
}

__global__ void __launch_bounds__(kSelectThreads) k_select(StepArgs a, int s, int sort_cap)
{
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ int s_cpref[kMaxChunks + 1];
    __shared__ uint32_t s_red[100];
    (void)sort_cap;
    const int seg = a.seg_lo + blockIdx.x;
    const SegDesc& d = a.segs[seg];
    if (threadIdx.x == 0) prefetch_desc(&d);
    pdl_wait();
    if (d.mode > MODE_CLEAN || s >= d.N) return;
    SegState& st = a.st[seg];
    const int P = st.P;   // issued with the prefix's loads
    const int nch = (d.K + a.chunk - 1) / a.chunk;
    uint32_t rmin, rmax;
    const int V = level_key_prefix(a, d, nch, s_cpref, s_red, rmin, rmax);
    if (threadIdx.x == 0) count_level(d.n, st, P, V);
    if (s == d.N - 1) return;  // the last level's sort and gather are not observable
    KeySrc ks;
    ks.base = a.keys + d.key_off;
    ks.cpref = s_cpref;
    ks.nch = nch;
    ks.cap = a.chunk * d.n;
    select_gpu(d, st, a, P, V, ks, smem, rmin, rmax);
}

// ---- cluster select: one beam's level on the C CTAs of a thread-block cluster ---------
// The bucket + dense-rank route of select_gpu with its data-parallel phases split: CTA r
// stages keys [r*V/C, (r+1)*V/C) of the level (slot order), builds its share of every
// histogram and table, and the CTAs exchange only small summaries through distributed
// shared memory (ld.shared::cluster of a peer's copy); the level's score range, and with it
// the bucket mapping, comes from the chunk ranges k_step records:
//   #1 the 4 096 bucket counts -> the same threshold bucket T in every CTA;
//   #2 the distinct-score bitmap (each CTA ORs the peers' words into its own; OR is
//      idempotent, so a peer reading a word before or after the merge sees the same
//      union) -> identical dense-rank tables;
//   #3 the per-digit survivor totals -> each survivor's global position
//      (digits below it in every CTA, its digit in lower CTAs, then its CTA's order).
// Every CTA scatters its survivors straight into the beam's survivor list.  With more
// distinct scores than kClusterMaxDigits, or a bitmap larger than kDenseWords, CTA 0
// gathers the survivors (its own, then the peers', which is slot order) and sorts them by
// LSD passes over the dense ranks or the raw score bits.  A level with more than kLsdMax
// survivors is left by all CTAs together after a cluster barrier and CTA 0 runs
// select_gpu on it; levels of at most kClusterMinKeys keys and forced one-CTA routes run
// there too.  A CTA only
// reads a peer's shared memory between two cluster barriers the peer also passes, and the
// last barrier before exit is split (arrive after the last remote read, wait before exit).
constexpr int kClusterMaxDigits = 1024;          // dense ranks of one counting pass (10 bits)
constexpr int kClusterTotOff = kDenseBmOff + kDenseWords;   // (in keys, after bitmap + prefix) i32 digit totals
constexpr int kClusterBaseOff = kClusterTotOff + kClusterMaxDigits / 2;   // i32[1024] digit bases
static_assert(32 * kClusterMaxDigits * 2 <= kDenseOccOff * 8, "per-warp digit counters must fit below the tables");
static_assert(kClusterBaseOff + kClusterMaxDigits / 2 <= kStageKeys, "cluster tables exceed the staging area");

__device__ __forceinline__ unsigned cluster_rank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// all threads of all CTAs of the cluster (release / acquire at cluster scope)
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_sync() { cluster_arrive(); cluster_wait(); }
// the shared-memory address of `p`'s counterpart in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t peer_addr(const void* p, unsigned rank)
{
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ uint32_t ld_peer(const void* p, unsigned rank)
{
    uint32_t v;
    asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(peer_addr(p, rank)) : "memory");
    return v;
}
__device__ __forceinline__ uint4 ld_peer4(const void* p, unsigned rank)
{
    uint4 v;
    asm volatile("ld.shared::cluster.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "r"(peer_addr(p, rank))
                 : "memory");
    return v;
}

// The gathered survivors A[0..count) (slot order) sorted by LSD passes over their dense
// ranks (D given) or score bits, the first R slots written to sel.  A separate function:
// its sort instantiations would otherwise spill the cluster route's registers.
__device__ __noinline__ void gathered_sort(unsigned long long* A, int count, int R, bool ranked, DenseTables D,
                                          uint32_t* sel, uint8_t* smem)
{
    const SelSmem S = sel_smem(smem);
    if (ranked) {
        for (int i = threadIdx.x; i < count; i += blockDim.x) {
            const unsigned long long k = A[i];
            A[i] = ((unsigned long long)D.rank_of((uint32_t)(k >> 32)) << 32) | (k & 0xFFFFFFFFull);
        }
        __syncthreads();
    }
    lsd_sort_emit_n(A, S.stg, count, R, sel, S);
}

// Returns the kPath* bits of the route when the level was selected (survivors 0..R-1
// written), 0 -- the same in every CTA, after a cluster barrier, nothing written -- when
// CTA 0 must run select_gpu.  On nonzero the caller still owes the closing cluster_wait().
template <int C>
__device__ uint32_t select_cluster(const KeySrc& ks, int V, int R, uint32_t* sel, const SelSmem& S, unsigned rank)
{
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;
    int* wsum = reinterpret_cast<int*>(S.red);
    const int lo = (int)((long long)V * rank / C), hi = (int)((long long)V * (rank + 1) / C);
    const int nl = hi - lo;   // <= kStageKeys: V <= C * kStageKeys
    unsigned long long* stg = S.stg;
    // 1. this CTA's keys, slot order, into stg (warp per chunk)
    for (int c = warp; c < ks.nch; c += nwarps) {
        const int c0 = ks.cpref[c];
        const int a0 = max(c0, lo), a1 = min(ks.cpref[c + 1], hi);
        const unsigned long long* src = ks.base + (size_t)c * ks.cap;
        for (int i = a0 + lane; i < a1; i += 32) cp_async8(stg + (i - lo), src + (i - c0));
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    // 2. bucket counts over the level's score range (from k_step's chunk ranges)
    uint32_t* cnt = S.hist;
    int* misc = S.misc;
    for (int b = tid; b < kNB; b += nthr) cnt[b] = 0;
    __syncthreads();
    const uint32_t smin = S.rmin, range = S.rmax - S.rmin;
    const int nbits = range ? 32 - __clz(range) : 0;
    const int shift = nbits > 12 ? nbits - 12 : 0;
    for (int i = tid; i < nl; i += nthr) atomicAdd(&cnt[bucket_of((uint32_t)(stg[i] >> 32), smin, shift)], 1u);
    cluster_sync();   // #1: every CTA's bucket counts (cnt, read by peers until #2)
    constexpr int BPT = kNB / kSelectThreads;
    static_assert(BPT == 4, "one 16-byte peer load per thread");
    uint32_t g4[BPT];
    {
        const uint4 own = *reinterpret_cast<const uint4*>(&cnt[tid * BPT]);
        g4[0] = own.x; g4[1] = own.y; g4[2] = own.z; g4[3] = own.w;
#pragma unroll
        for (int q = 0; q < C; q++) {
            if (q == (int)rank) continue;
            const uint4 v = ld_peer4(&cnt[tid * BPT], q);
            g4[0] += v.x; g4[1] += v.y; g4[2] += v.z; g4[3] += v.w;
        }
    }
    int sum = 0;
#pragma unroll
    for (int u = 0; u < BPT; u++) sum += (int)g4[u];
    int tot;
    int base = block_exclusive_scan(sum, &tot, wsum);
#pragma unroll
    for (int u = 0; u < BPT; u++) {
        if (base < R && R <= base + (int)g4[u]) { misc[2] = tid * BPT + u; misc[3] = base + (int)g4[u]; }
        base += (int)g4[u];
    }
    __syncthreads();
    const int T = misc[2], count = misc[3];   // survivors: the keys of buckets <= T, cluster-wide
    if (count > kLsdMax) { cluster_sync(); return 0u; }
    // 3. this CTA's survivors, stably compacted into A
    const uint32_t lim = ((uint32_t)T + 1u) << shift;
    auto keep = [=](unsigned long long k) { return (((uint32_t)(k >> 32)) - smin) < lim; };
    auto get_s = [=](int i) { return stg[i]; };
    unsigned long long* A = S.A;
    const int cl = compact_stable(get_s, nl, keep, A, kLsdMax, S);
    // 4. dense-rank tables (stg is free now): occupied-bucket index from the cluster's
    // counts, this CTA's bits, then the union of the CTAs' bitmaps
    DenseTables D;
    D.occ = reinterpret_cast<uint16_t*>(stg + kDenseOccOff);
    D.bm = reinterpret_cast<uint32_t*>(stg + kDenseBmOff);
    D.wp = D.bm + kDenseWords;
    D.W = shift > 5 ? 1 << (shift - 5) : 1;
    D.shift = shift;
    D.smin = smin;
    D.omask = (1u << shift) - 1u;
    int f[BPT], fs = 0;
#pragma unroll
    for (int u = 0; u < BPT; u++) {
        f[u] = (tid * BPT + u <= T && g4[u] != 0u) ? 1 : 0;
        fs += f[u];
    }
    int O;
    int ob = block_exclusive_scan(fs, &O, wsum);
#pragma unroll
    for (int u = 0; u < BPT; u++) {
        D.occ[tid * BPT + u] = (uint16_t)ob;
        ob += f[u];
    }
    const int nw = O * D.W;   // the same in every CTA
    int nd = -1;
    if (nw <= kDenseWords) {
        for (int w = tid; w < nw; w += nthr) D.bm[w] = 0u;
        __syncthreads();
        for (int i = tid; i < cl; i += nthr) {
            uint32_t bit;
            const int w = D.word_of((uint32_t)(A[i] >> 32), bit);
            atomicOr(&D.bm[w], 1u << bit);
        }
        cluster_sync();   // #2: every CTA's bitmap (read by peers until #3); cnt is free again
        const int per = (nw + nthr - 1) / nthr;
        int pc = 0;
        for (int k = 0; k < per; k++) {
            const int w = tid * per + k;
            if (w < nw) {
                uint32_t v = D.bm[w];
#pragma unroll
                for (int q = 0; q < C; q++)
                    if (q != (int)rank) v |= ld_peer(&D.bm[w], q);
                D.bm[w] = v;
                pc += __popc(v);
            }
        }
        int pre = block_exclusive_scan(pc, &nd, wsum);
        for (int k = 0; k < per; k++) {
            const int w = tid * per + k;
            if (w < nw) {
                D.wp[w] = (uint32_t)pre;
                pre += __popc(D.bm[w]);
            }
        }
    }
    if (nd < 0 || nd > kClusterMaxDigits) {   // the same in every CTA
        // too many distinct scores for one counting pass (or no tables): CTA 0 gathers the
        // survivors -- its own, then each peer's, which is slot order -- and sorts them with
        // LSD passes (over the dense ranks when the tables exist, else the score bits)
        if (tid == 0) misc[5] = cl;
        cluster_sync();   // every CTA's survivors and count (misc[5]); bitmap merges done
        if (rank == 0) {
            int off = cl;
            for (int q = 1; q < C; q++) {
                const int cq = (int)ld_peer(&misc[5], q);
                for (int i = tid; i < cq; i += nthr) {
                    const uint32_t* pk = reinterpret_cast<const uint32_t*>(&A[i]);
                    const uint32_t lo32 = ld_peer(pk, q), hi32 = ld_peer(pk + 1, q);
                    A[off + i] = ((unsigned long long)hi32 << 32) | lo32;
                }
                off += cq;
            }
        }
        cluster_arrive();  // CTA 0's remote reads are done
        if (rank == 0) {
            __syncthreads();
            gathered_sort(A, count, R, nd >= 0, D, sel, reinterpret_cast<uint8_t*>(S.hist));
        }
        return kPathCluster | (nd >= 0 ? kPathRankLsd : kPathRawLsd);
    }
    // 5. one stable counting pass by dense rank: per-warp digit counters (u16 [32][ND] over
    // the start of stg), ranks found with bit ballots, element order within the warp
    const int db = nd > 1 ? 32 - __clz(nd - 1) : 1;
    const int ND = 1 << db;
    uint16_t* wh = reinterpret_cast<uint16_t*>(stg);
    int* dtot = reinterpret_cast<int*>(stg + kClusterTotOff);
    int* dbase = reinterpret_cast<int*>(stg + kClusterBaseOff);
    for (int i = tid; i < 32 * ND / 2; i += nthr) reinterpret_cast<uint32_t*>(wh)[i] = 0u;
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    const int E = (cl + nthr - 1) / nthr;
#pragma unroll 1
    for (int e = 0; e < E; e++) {
        const int p = warp * 32 * E + e * 32 + lane;
        const bool valid = p < cl;
        const unsigned long long x = valid ? A[p] : 0ull;
        const int d = valid ? (int)D.rank_of((uint32_t)(x >> 32)) : 0;
        unsigned grp = __ballot_sync(FULL_MASK, valid);
#pragma unroll 1
        for (int bit = 0; bit < db; bit++) {
            const unsigned bb = __ballot_sync(FULL_MASK, (d >> bit) & 1);
            grp &= ((d >> bit) & 1) ? bb : ~bb;
        }
        const int r_in = __popc(grp & lt);
        int b = 0;
        if (valid) b = wh[warp * ND + d];
        __syncwarp();
        if (valid && r_in == 0) wh[warp * ND + d] = (uint16_t)(b + __popc(grp));
        __syncwarp();
        if (valid)
            A[p] = ((unsigned long long)d << 48) | ((unsigned long long)(b + r_in) << 32) | (x & 0xFFFFFFFFull);
    }
    __syncthreads();
    if (tid < ND) {
        int run = 0;
        for (int w = 0; w < nwarps; w++) {
            const int t = wh[w * ND + tid];
            wh[w * ND + tid] = (uint16_t)run;
            run += t;
        }
        dtot[tid] = run;
    }
    cluster_sync();   // #3: every CTA's digit totals (read by peers until the closing wait)
    // the level's last ~2 us: let the next k_step's launch start now, so its CTAs are resident
    // when this grid completes (8-beam bench -0.35 %; triggering after #2 gained nothing)
    pdl_trigger();
    int g = 0, lower = 0;
    if (tid < ND) {
#pragma unroll
        for (int q = 0; q < C; q++) {
            const int t = q == (int)rank ? dtot[tid] : (int)ld_peer(&dtot[tid], q);
            g += t;
            if (q < (int)rank) lower += t;
        }
    }
    cluster_arrive();  // this CTA's remote reads are done
    int gt;
    const int gb = block_exclusive_scan(g, &gt, wsum);
    if (tid < ND) dbase[tid] = gb + lower;
    __syncthreads();
#pragma unroll 1
    for (int e = 0; e < E; e++) {
        const int p = warp * 32 * E + e * 32 + lane;
        if (p < cl) {
            const unsigned long long x = A[p];
            const int dg = (int)(x >> 48);
            const int pos = dbase[dg] + (int)wh[warp * ND + dg] + (int)((x >> 32) & 0xFFFFull);
            if (pos < R) sel[pos] = (uint32_t)(x & 0xFFFFFFFFull);
        }
    }
    return kPathCluster;
}

// the one-CTA routes as a separate function: the cluster kernel's registers stay for its own route
__device__ __noinline__ void select_gpu_fallback(const SegDesc& d, SegState& st, const StepArgs& a, int P, int V,
                                                 const KeySrc& ks, uint8_t* smem, uint32_t rmin, uint32_t rmax)
{
    select_gpu(d, st, a, P, V, ks, smem, rmin, rmax);
}

// k_select launched as clusters of C CTAs per beam (blocks C*b .. C*b+C-1 serve beam
// seg_lo + b).  Levels the cluster route takes run on all C CTAs; the rest run select_gpu
// on CTA 0 while the others leave.
template <int C>
__global__ void __launch_bounds__(kSelectThreads) k_select_cl(StepArgs a, int s, int sort_cap)
{
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ int s_cpref[kMaxChunks + 1];
    __shared__ uint32_t s_red[100];
    (void)sort_cap;
    const unsigned rank = cluster_rank();
    const int seg = a.seg_lo + (int)(blockIdx.x / C);
    const SegDesc& d = a.segs[seg];
    if (threadIdx.x == 0) prefetch_desc(&d);
    pdl_wait();
    if (d.mode > MODE_CLEAN || s >= d.N) return;   // the same for the whole cluster
    SegState& st = a.st[seg];
    const int P = st.P;   // issued with the prefix's loads
    const int nch = (d.K + a.chunk - 1) / a.chunk;
    uint32_t rmin, rmax;
    const int V = level_key_prefix(a, d, nch, s_cpref, s_red, rmin, rmax);
    const int K = d.K;
    if (rank == 0 && threadIdx.x == 0) count_level(d.n, st, P, V);
    if (s == d.N - 1) return;  // the last level's sort and gather are not observable
    KeySrc ks;
    ks.base = a.keys + d.key_off;
    ks.cpref = s_cpref;
    ks.nch = nch;
    ks.cap = a.chunk * d.n;
    const int total = P * d.n;
    const int keff = (d.mode == MODE_CLEAN) ? (V < K ? V : K) : (total < K ? total : K);
    const int R = V < keff ? V : keff;
    const int fz = a.select_force;
    const bool take = (fz & ~kSelForceCluster) == 0 && R > 0 && K <= kLsdMax && V <= C * kStageKeys &&
                      ((fz & kSelForceCluster) || V > kClusterMinKeys);
    uint32_t* sel = a.sel + d.sel_off;
    const uint32_t path = take ? select_cluster<C>(ks, V, R, sel, sel_smem(smem, rmin, rmax), rank) : 0u;
    if (path) {
        if (rank == 0) {
            if (threadIdx.x == 0) atomicOr(&st.select_paths, path);
            __syncthreads();
            select_fillers(d, a, P, R, keff, sel, smem);
            __syncthreads();
            if (threadIdx.x == 0) {
                st.P = keff;
                atomicAdd(reinterpret_cast<unsigned long long*>(&st.materialized), (unsigned long long)keff);
            }
        }
        cluster_wait();   // peers may read this CTA's digit totals until here
        return;
    }
    if (rank == 0) select_gpu_fallback(d, st, a, P, V, ks, smem, rmin, rmax);
}

// ------------------------------------------------------------------------------------
// k_heap: ICH / PMS selection per beam, in the CPU solvers' order (cpu/v0_ich/solver.cpp:
// 22-39, cpu/v1_pms/solver.cpp:26-62, insert_into_beam jssp_types.h:47-58).
//
// The survivors and their order (the next level's parent order) are what libstdc++'s
// bounded heap holds after every child has been offered in generation order, so the heap
// stays serial: lane 0 of warp 0 runs it and nothing else.  Warps 1..7 work one chunk of
// parents ahead of it:
//   1. stage the chunk's child tables (written by k_step) in shared memory;
//   2. consume the glibc rand() stream.  ICH draws one value per child, so the chunk's
//      draws are known in advance and one warp generates them 31 at a time
//      (warp_rand_fill).  BS-PMS draws a pivot and then one value per child on the pivot's
//      machine, so one lane walks the parents, reading each position's machine count from
//      a table the warps built with a histogram per parent;
//   3. score every child (thread per child) and drop those the heap would reject anyway:
//      once the heap is full its front only decreases, so a key that is not below a front
//      published earlier is not below the front when its turn comes;
//   4. compact the remaining children, in generation order, into the buffer the heap
//      thread reads on its next pass.
// ------------------------------------------------------------------------------------
constexpr int kHeapProducers = kHeapThreads - 32;
constexpr int kHeapProducerWarps = kHeapProducers / 32;
constexpr int kHeapMiscBytes = 128 + kHeapProducerWarps * 64 * 4;

__host__ __device__ __forceinline__ size_t hl_align(size_t x) { return (x + 15) & ~(size_t)15; }

// hk [K] u64 | hv [K] u32 | misc | per-parent coff [C+1], pm [C], rbase [C] | rb [34 + C(n+1)]
// u32 | stage [C] child tables | cpar, cpos [C n] u8 | cdraw [C n] u32 | cntv [C n] u8 |
// ck [2][C n] u64 | cv [2][C n] u32
struct HeapLayout {
    size_t hk, hv, misc, pp, rb, stage, cpar, cpos, cdraw, cntv, ck, cv, total;
    __host__ __device__ explicit HeapLayout(const HeapCfg& c)
    {
        const size_t C = (size_t)c.chunk, cap = (size_t)c.chunk * (size_t)c.nmax;
        size_t o = 0;
        hk = o;
        o += 8 * (size_t)c.kmax;
        hv = o;
        o = hl_align(o + 4 * (size_t)c.kmax);
        misc = o;
        o += kHeapMiscBytes;
        pp = o;
        o = hl_align(o + 4 * (3 * C + 1));
        rb = o;
        o = hl_align(o + 4 * (34 + C * ((size_t)c.nmax + 1)));
        stage = o;
        o = hl_align(o + C * (size_t)c.ab);
        cpar = o;
        o = hl_align(o + cap);
        cpos = o;
        o = hl_align(o + cap);
        cdraw = o;
        o = hl_align(o + 4 * cap);
        cntv = o;
        o = hl_align(o + cap);
        ck = o;
        o += 2 * 8 * cap;
        cv = o;
        o = hl_align(o + 2 * 4 * cap);
        total = o;
    }
};

size_t heap_smem_bytes(const HeapCfg& c) { return HeapLayout(c).total; }

int heap_pick_chunk(HeapCfg c, size_t budget)
{
    for (int ch = kHeapMaxChunk; ch >= 1; ch--) {
        c.chunk = ch;
        if (heap_smem_bytes(c) <= budget) return ch;
    }
    return 0;
}

// libstdc++ __push_heap: the value rises from `hole` while its parent is smaller.  The
// parent's value is loaded with its key, so a move costs one shared-memory round trip.
__device__ __forceinline__ void heap_sift_up(unsigned long long* hk, uint32_t* hv, int hole, int top,
                                             unsigned long long vk, uint32_t vv)
{
    while (hole > top) {
        const int parent = (hole - 1) / 2;
        const unsigned long long kp = hk[parent];
        const uint32_t vp = hv[parent];
        if (!(kp < vk)) break;
        hk[hole] = kp;
        hv[hole] = vp;
        hole = parent;
    }
    hk[hole] = vk;
    hv[hole] = vv;
}

// libstdc++ __adjust_heap: the hole walks down to a leaf along the larger children (the
// right one on ties, a lone left child is taken), then the value is pushed up from there.
// Both children's keys and values are loaded together, so each level of the walk costs
// one shared-memory round trip (the value no longer waits for the comparison).  (Loading
// the four grandchildren as well, two levels per round, measured slower: 4.94 vs 4.64 s
// per 8-beam BS-PMS search at 50x20, K=4096 -- the heap thread is issue-bound by then.)
__device__ void heap_adjust(unsigned long long* hk, uint32_t* hv, int hole, int len,
                            unsigned long long vk, uint32_t vv)
{
    const int top = hole;
    int child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        const unsigned long long kr = hk[child], kl = hk[child - 1];
        const uint32_t vr = hv[child], vl = hv[child - 1];
        const bool left = kr < kl;
        child -= left ? 1 : 0;
        hk[hole] = left ? kl : kr;
        hv[hole] = left ? vl : vr;
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        hk[hole] = hk[child - 1];
        hv[hole] = hv[child - 1];
        hole = child - 1;
    }
    heap_sift_up(hk, hv, hole, top, vk, vv);
}

// glibc rand() (TYPE_3): r[t] = r[t-31] + r[t-3] mod 2^32, rand() = r[t] >> 1.
// rb[0..34) hold r[t0-34 .. t0-1]; writes r[t0 .. t0+cnt) to rb[34 ..).  Lane j makes
// r[t+j] for 31 positions per step: unrolled, r[t+j] = sum over k of r[t+j-31-3k] (a
// stride-3 inclusive prefix sum of the lanes' x_j = r[t+j-31]) + r[t-3+(j mod 3)].
__device__ void warp_rand_fill(uint32_t* rb, int cnt, int lane)
{
    uint32_t x = lane < 31 ? rb[3 + lane] : 0u;
    uint32_t b = rb[31 + lane % 3];
    for (int t = 0; t < cnt; t += 31) {
        uint32_t v = x, u;
        u = __shfl_up_sync(FULL_MASK, v, 3);
        if (lane >= 3) v += u;
        u = __shfl_up_sync(FULL_MASK, v, 6);
        if (lane >= 6) v += u;
        u = __shfl_up_sync(FULL_MASK, v, 12);
        if (lane >= 12) v += u;
        u = __shfl_up_sync(FULL_MASK, v, 24);
        if (lane >= 24) v += u;
        v += b;
        if (lane < 31 && t + lane < cnt) rb[34 + t + lane] = v;
        x = v;
        b = __shfl_sync(FULL_MASK, v, 28 + lane % 3);
    }
}

__global__ void __launch_bounds__(kHeapThreads) k_heap(StepArgs a, int s, HeapCfg cfg)
{
    pdl_wait();
    extern __shared__ __align__(16) uint8_t smem[];
    const int seg = a.seg_lo + blockIdx.x;
    const SegDesc& d = a.segs[seg];
    if (d.mode < MODE_ICH || s >= d.N) return;
    SegState& st = a.st[seg];
    const HeapLayout HL(cfg);
    unsigned long long* hk = reinterpret_cast<unsigned long long*>(smem + HL.hk);
    uint32_t* hv = reinterpret_cast<uint32_t*>(smem + HL.hv);
    uint8_t* misc = smem + HL.misc;
    unsigned long long* s_front = reinterpret_cast<unsigned long long*>(misc);      // published heap front
    unsigned long long* s_best = reinterpret_cast<unsigned long long*>(misc + 8);   // (cmax << 32 | ref) min
    int* s_cnt = reinterpret_cast<int*>(misc + 16);                                 // [2] kept children
    int* s_wsum = reinterpret_cast<int*>(misc + 24);                                // [8] per-warp counts
    int* s_dtot = reinterpret_cast<int*>(misc + 56);                                // draws so far
    int* s_draws = reinterpret_cast<int*>(misc + 60);                               // draws of a chunk
    int* s_size = reinterpret_cast<int*>(misc + 64);
    uint32_t* hist = reinterpret_cast<uint32_t*>(misc + 128);                       // [warps][64]
    const int C = cfg.chunk;
    int* coff = reinterpret_cast<int*>(smem + HL.pp);  // [C+1] first child of each parent
    int* pm = coff + C + 1;                            // [C] BS-PMS pivot machine
    int* rbase = pm + C;                               // [C] BS-PMS first noise draw (rb index)
    uint32_t* rb = reinterpret_cast<uint32_t*>(smem + HL.rb);
    uint8_t* stage = smem + HL.stage;
    uint8_t* cpar = smem + HL.cpar;
    uint8_t* cpos = smem + HL.cpos;
    uint32_t* cdraw = reinterpret_cast<uint32_t*>(smem + HL.cdraw);
    uint8_t* cntv = smem + HL.cntv;
    const size_t cap = (size_t)C * cfg.nmax;
    unsigned long long* ck = reinterpret_cast<unsigned long long*>(smem + HL.ck);
    uint32_t* cv = reinterpret_cast<uint32_t*>(smem + HL.cv);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int K = d.K, n = d.n, ab = d.auxbytes;
    const int P = st.P;
    const uint8_t* aux = a.aux_pool + d.aux_off;
    const bool ich = (d.mode == MODE_ICH);
    const bool last = (s == d.N - 1);
    const int bound = st.bound;
    const uint32_t k0 = st.rng_i - 34u;
    const int nchunks = (P + C - 1) / C;
    if (tid == 0) {
        *s_front = ~0ull;
        *s_best = ~0ull;
        *s_dtot = 0;
    }
    if (tid < 34) rb[tid] = st.rng[(k0 + (uint32_t)tid) % 34u];
    __syncthreads();

    const int pt = tid - 32, pw = warp - 1;
    long long gen = 0;
    auto pbar = [] { asm volatile("bar.sync 1, %0;" ::"r"(kHeapProducers) : "memory"); };
    auto produce = [&](int q) {
        if (q >= nchunks) return;
        const int c0 = q * C;
        const int cnt = (P - c0) < C ? (P - c0) : C;
        {
            const uint4* s4 = reinterpret_cast<const uint4*>(aux + (int64_t)c0 * ab);
            uint4* d4 = reinterpret_cast<uint4*>(stage);
            for (int u = pt; u < (cnt * ab) >> 4; u += kHeapProducers) d4[u] = __ldcg(s4 + u);
        }
        pbar();
        auto rc_of = [&](int p) { return (int)*reinterpret_cast<const uint32_t*>(stage + (size_t)p * ab); };
        auto cc_of = [&](int p) { return reinterpret_cast<const int32_t*>(stage + (size_t)p * ab + 4); };
        auto mc_of = [&](int p) { return stage + (size_t)p * ab + 4 + 4 * n; };
        if (ich) {
            if (pw == 0) {
                // cpu/v0_ich/solver.cpp:22-35: one draw per child, parents in order
                const int v = lane < cnt ? rc_of(lane) : 0;
                int x = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(FULL_MASK, x, o);
                    if (lane >= o) x += y;
                }
                if (lane < cnt) coff[lane] = x - v;
                const int T = __shfl_sync(FULL_MASK, x, 31);
                if (lane == 0) {
                    coff[cnt] = T;
                    *s_draws = T;
                }
                warp_rand_fill(rb, T, lane);
            }
            pbar();
        } else {
            // machines' ready-op counts per ready position (histogram per parent)
            uint32_t* wh = hist + pw * 64;
            for (int p = pw; p < cnt; p += kHeapProducerWarps) {
                const int rc = rc_of(p);
                const uint8_t* mc = mc_of(p);
                wh[lane] = 0;
                wh[lane + 32] = 0;
                __syncwarp();
                for (int i = lane; i < rc; i += 32) atomicAdd(&wh[mc[i]], 1u);
                __syncwarp();
                for (int i = lane; i < rc; i += 32) cntv[p * n + i] = (uint8_t)wh[mc[i]];
                __syncwarp();
            }
            pbar();
            if (pt == 0) {
                // cpu/v1_pms/solver.cpp:26-53: a parent with ready ops draws its pivot, then one
                // noise value per ready op on the pivot's machine, in ready-list order
                int pos = 34, k = 0;
                uint32_t r3 = rb[31], r2 = rb[32], r1 = rb[33];
                for (int p = 0; p < cnt; p++) {
                    const int rc = rc_of(p);
                    coff[p] = k;
                    rbase[p] = pos;
                    if (rc == 0) {
                        pm[p] = -1;
                        continue;
                    }
                    uint32_t v = rb[pos - 31] + r3;
                    rb[pos++] = v;
                    r3 = r2; r2 = r1; r1 = v;
                    const int piv = (int)((v >> 1) % (uint32_t)rc);
                    pm[p] = mc_of(p)[piv];
                    const int c = cntv[p * n + piv];
                    rbase[p] = pos;
                    for (int j = 0; j < c; j++) {
                        v = rb[pos - 31] + r3;
                        rb[pos++] = v;
                        r3 = r2; r2 = r1; r1 = v;
                    }
                    k += c;
                }
                coff[cnt] = k;
                *s_draws = pos - 34;
            }
            pbar();
        }
        const int T = coff[cnt];
        const int D = *s_draws;
        // children in generation order: parent, ready position, its draw
        for (int p = pw; p < cnt; p += kHeapProducerWarps) {
            const int rc = rc_of(p);
            const int base = coff[p];
            if (ich) {
                for (int i = lane; i < rc; i += 32) {
                    const int k = base + i;
                    cpar[k] = (uint8_t)p;
                    cpos[k] = (uint8_t)i;
                    cdraw[k] = rb[34 + k];
                }
            } else {
                const int pmach = pm[p];
                const uint8_t* mc = mc_of(p);
                const int r0 = rbase[p];
                int carry = 0;
                for (int i0 = 0; i0 < rc; i0 += 32) {
                    const int i = i0 + lane;
                    const bool on = i < rc && (int)mc[i] == pmach;
                    const uint32_t bal = __ballot_sync(FULL_MASK, on);
                    if (on) {
                        const int r = carry + __popc(bal & ((1u << lane) - 1u));
                        cpar[base + r] = (uint8_t)p;
                        cpos[base + r] = (uint8_t)i;
                        cdraw[base + r] = rb[r0 + r];
                    }
                    carry += __popc(bal);
                }
            }
        }
        pbar();
        // score, drop what the heap would reject, compact in order
        const double ns = (double)(s + 1);
        unsigned long long bmin = ~0ull;
        unsigned long long* okey = ck + (size_t)(q & 1) * cap;
        uint32_t* oval = cv + (size_t)(q & 1) * cap;
        int out = 0;
        for (int t0 = 0; t0 < T; t0 += kHeapProducers) {
            const int k = t0 + pt;
            bool keep = false;
            unsigned long long key = 0;
            uint32_t val = 0;
            if (k < T) {
                const int p = cpar[k], i = cpos[k];
                const int cc = cc_of(p)[i];
                const uint32_t dr = cdraw[k] >> 1;
                const unsigned long long F = *reinterpret_cast<volatile unsigned long long*>(s_front);
                if (ich) {
                    // score = cmax + (rand()%100)*0.01 (cpu/v0_ich/solver.cpp:35): the pair
                    // (cmax, rand()%100) orders exactly like that double
                    key = (unsigned long long)cc * 100ull + (dr % 100u);
                    keep = key < F;
                } else {
                    // cpu/v1_pms/solver.cpp:52-57
                    const double sc = __dadd_rn(__ddiv_rn((double)cc, ns), a.dnoise[dr % 1000u]);
                    key = (unsigned long long)__double_as_longlong(sc);
                    keep = cc < bound && key < F;
                    if (last && cc < kSentinel) {
                        const unsigned long long bk = ((unsigned long long)(uint32_t)cc << 32) |
                                                      ((unsigned long long)(c0 + p) << 8) | (unsigned)i;
                        bmin = bk < bmin ? bk : bmin;
                    }
                }
                val = ((uint32_t)(c0 + p) << 8) | (uint32_t)i;
            }
            const uint32_t bal = __ballot_sync(FULL_MASK, keep);
            if (lane == 0) s_wsum[pw] = __popc(bal);
            pbar();
            int off = out, tot = 0;
#pragma unroll
            for (int w = 0; w < kHeapProducerWarps; w++) {
                const int x = s_wsum[w];
                off += (w < pw) ? x : 0;
                tot += x;
            }
            if (keep) {
                const int o = off + __popc(bal & ((1u << lane) - 1u));
                okey[o] = key;
                oval[o] = val;
            }
            out += tot;
            pbar();
        }
        if (last && !ich) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long y = __shfl_xor_sync(FULL_MASK, bmin, o);
                bmin = y < bmin ? y : bmin;
            }
            if (lane == 0 && bmin != ~0ull) atomicMin(s_best, bmin);
        }
        if (pt == 0) {
            s_cnt[q & 1] = out;
            gen += T;
        }
        // the stream's last 34 values are the next chunk's history
        const uint32_t hold = pt < 34 ? rb[D + pt] : 0u;
        pbar();
        if (pt < 34) rb[pt] = hold;
        if (pt == 0) *s_dtot += D;
    };

    if (warp > 0) produce(0);
    __syncthreads();
    int size = 0;
    unsigned long long front = ~0ull;
    for (int q = 0; q < nchunks; q++) {
        if (warp > 0) {
            produce(q + 1);
        } else if (lane == 0) {
            // insert_into_beam (jssp_types.h:47-58): push while below K, else replace the
            // front (pop_heap, overwrite the back, push_heap) when strictly better
            const int nc = s_cnt[q & 1];
            const unsigned long long* ik = ck + (size_t)(q & 1) * cap;
            const uint32_t* iv = cv + (size_t)(q & 1) * cap;
            unsigned long long nkey = nc > 0 ? ik[0] : 0ull;
            uint32_t nval = nc > 0 ? iv[0] : 0u;
            for (int k = 0; k < nc; k++) {
                const unsigned long long key = nkey;
                const uint32_t val = nval;
                if (k + 1 < nc) {
                    nkey = ik[k + 1];
                    nval = iv[k + 1];
                }
                if (size < K) {
                    heap_sift_up(hk, hv, size, 0, key, val);
                    if (++size == K) {
                        front = hk[0];
                        *reinterpret_cast<volatile unsigned long long*>(s_front) = front;
                    }
                } else if (key < front) {
                    if (size > 1) heap_adjust(hk, hv, 0, size - 1, hk[size - 1], hv[size - 1]);
                    heap_sift_up(hk, hv, size - 1, 0, key, val);
                    front = hk[0];
                    *reinterpret_cast<volatile unsigned long long*>(s_front) = front;
                }
            }
            *s_size = size;
        }
        __syncthreads();
    }
    if (nchunks == 0 && tid == 0) *s_size = 0;
    if (tid == 32) {
        st.expanded += gen;
        st.slots += gen;
    }
    if (last && ich) {
        // min makespan over the final beam, first in array order (cpu/v0_ich/solver.cpp:47-51)
        __syncthreads();
        const int fs = *s_size;
        unsigned long long bmin = ~0ull;
        for (int r = tid; r < fs; r += blockDim.x) {
            const uint32_t e = hv[r];
            const uint8_t* pa = aux + (int64_t)(e >> 8) * ab;
            const int cm = reinterpret_cast<const int32_t*>(pa + 4)[e & 0xFFu];
            if (cm < kSentinel) {
                const unsigned long long bk = ((unsigned long long)(uint32_t)cm << 32) | (unsigned)r;
                bmin = bk < bmin ? bk : bmin;
            }
        }
        if (bmin != ~0ull) atomicMin(s_best, bmin);
    }
    __syncthreads();
    const int out_size = *s_size;
    if (tid == 0) {
        const uint32_t dt = (uint32_t)*s_dtot;
        st.rng_i = 34u + (k0 + dt) % 34u;
        if (P > 0) st.levels += 1;
        st.P = out_size;
        if (!last) st.materialized += out_size;
        if (last) {
            int best_cm = kSentinel;
            uint32_t best_ref = 0;
            const unsigned long long b = *s_best;
            if (b != ~0ull) {
                best_cm = (int)(b >> 32);
                uint32_t c, i;
                if (ich) {
                    const uint32_t e = hv[(uint32_t)b];
                    c = e >> 8;
                    i = e & 0xFFu;
                } else {
                    c = (uint32_t)(b >> 8) & 0xFFFFFFu;
                    i = (uint32_t)b & 0xFFu;
                }
                best_ref = (c << 8) | (uint32_t)aux[(int64_t)c * ab + 4 + 5 * n + i];
            }
            st.best_cmax = best_cm;
            st.best_ref = best_ref;
        }
    }
    if (tid < 34) st.rng[(k0 + (uint32_t)*s_dtot + (uint32_t)tid) % 34u] = rb[tid];
    uint32_t* sel = a.sel + d.sel_off;
    for (int r = tid; r < out_size; r += blockDim.x) sel[r] = hv[r];
}

// ------------------------------------------------------------------------------------
// k_finalize: result makespan and the best schedule rebuilt from the level history.
// ------------------------------------------------------------------------------------
__global__ void k_finalize(StepArgs a)
{
    const int seg = blockIdx.x * blockDim.x + threadIdx.x;
    if (seg >= a.nseg) return;
    const SegDesc& d = a.segs[seg];
    SegState& st = a.st[seg];
    int32_t* seq = a.seq_pool + d.seq_off;
    const int N = d.N;
    bool found = false;
    int mk = kSentinel;
    int c = 0, job = 0;
    if (d.mode <= MODE_CLEAN) {
        mk = st.bound;
        if (st.best != ~0ull) {
            const int cm = (int)(st.best >> 32);
            const uint32_t slot = (uint32_t)((st.best >> 8) & 0xFFFFFFull);
            job = (int)(st.best & 0xFFull);
            c = (int)(slot / (uint32_t)d.n);
            found = true;
            mk = cm < mk ? cm : mk;
        }
    } else {
        mk = st.best_cmax;
        if (st.best_cmax < kSentinel) {
            found = true;
            c = (int)(st.best_ref >> 8);
            job = (int)(st.best_ref & 0xFFu);
        }
    }
    if (found && (c >= d.K || job >= d.n)) {
        found = false;
        atomicOr(&st.status, kStatusBadLineage);
    }
    if (found) {
        seq[N - 1] = job;
        for (int t = N - 2; t >= 0; t--) {
            const uint32_t e = a.hist[d.hist_off + (int64_t)t * d.K + c];
            if (e == kMark || (int)(e >> 8) >= d.K || (int)(e & 0xFFu) >= d.n) {
                found = false;
                atomicOr(&st.status, kStatusBadLineage);
                break;
            }
            seq[t] = (int)(e & 0xFFu);
            c = (int)(e >> 8);
        }
    }
    if (found) {
        int cnt[kMaxJobs];
        for (int j = 0; j < d.n; j++) cnt[j] = 0;
        for (int t = 0; t < N; t++) {
            const int j = seq[t];
            seq[t] = j * d.m + cnt[j] + 1;
            cnt[j]++;
        }
    } else {
        for (int t = 0; t < N; t++) seq[t] = 0;
    }
    st.makespan = mk;
    st.found = found ? 1 : 0;
}

// ------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------
size_t step_smem_bytes(int sb_max, int max_n, int chunk)
{
    return (size_t)kWarpsPerStepCta * (chunk / kWarpsPerStepCta + 1) * sb_max + (size_t)chunk * max_n * 8;
}

// every k_step instantiation: NQ in {1, 2, 4} x chunk in kChunkSizes
template <typename F>
static cudaError_t for_each_step(F&& f)
{
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = f(k_step<1, 8>, 8);
    if (e == cudaSuccess) e = f(k_step<2, 8>, 8);
    if (e == cudaSuccess) e = f(k_step<4, 8>, 8);
    if (e == cudaSuccess) e = f(k_step<1, 16>, 16);
    if (e == cudaSuccess) e = f(k_step<2, 16>, 16);
    if (e == cudaSuccess) e = f(k_step<4, 16>, 16);
    if (e == cudaSuccess) e = f(k_step<1, 32>, 32);
    if (e == cudaSuccess) e = f(k_step<2, 32>, 32);
    if (e == cudaSuccess) e = f(k_step<4, 32>, 32);
    return e;
}

template <typename F>
static cudaError_t for_each_gstep(F&& f)
{
    cudaError_t e = f(k_step_g<4, 1>, 4);
    if (e == cudaSuccess) e = f(k_step_g<4, 2>, 4);
    if (e == cudaSuccess) e = f(k_step_g<8, 1>, 8);
    if (e == cudaSuccess) e = f(k_step_g<8, 2>, 8);
    return e;
}

int nq_class(int n) { return n <= 32 ? 1 : (n <= 64 ? 2 : 4); }

// All level kernels run back to back; giving them one shared-memory carveout (the
// maximum) keeps the SMs from being reconfigured between k_select and k_step.
static cudaError_t set_carveout()
{
    const int c = cudaSharedmemCarveoutMaxShared;
    cudaError_t e = cudaFuncSetAttribute(k_select, cudaFuncAttributePreferredSharedMemoryCarveout, c);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_select_cl<2>, cudaFuncAttributePreferredSharedMemoryCarveout, c);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_select_cl<4>, cudaFuncAttributePreferredSharedMemoryCarveout, c);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_heap, cudaFuncAttributePreferredSharedMemoryCarveout, c);
    if (e == cudaSuccess)
        e = for_each_step([&](auto fn, int) { return cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, c); });
    if (e == cudaSuccess)
        e = for_each_gstep([&](auto fn, int) { return cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, c); });
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_gather_v1, cudaFuncAttributePreferredSharedMemoryCarveout, c);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_finalize, cudaFuncAttributePreferredSharedMemoryCarveout, c);
    return e;
}

// The dynamic shared-memory limit is an attribute of the kernel, shared by every plan,
// context and thread of the process, and graphs captured earlier launch with the sizes
// they were captured with: limits are only ever raised, under one lock.
static std::mutex g_attr_mu;

template <typename F>
static cudaError_t raise_smem(F* fn, size_t bytes)
{
    cudaFuncAttributes at;
    cudaError_t e = cudaFuncGetAttributes(&at, fn);
    if (e != cudaSuccess) return e;
    if ((size_t)at.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

cudaError_t configure_kernels(int sort_cap, const HeapCfg* hc, int sb_max, int max_n)
{
    std::lock_guard<std::mutex> lk(g_attr_mu);
    cudaError_t e = set_carveout();
    if (e == cudaSuccess) e = raise_smem(k_select, select_smem_bytes(sort_cap));
    if (e == cudaSuccess) e = raise_smem(k_select_cl<2>, select_smem_bytes(sort_cap));
    if (e == cudaSuccess) e = raise_smem(k_select_cl<4>, select_smem_bytes(sort_cap));
    if (e == cudaSuccess && hc) e = raise_smem(k_heap, heap_smem_bytes(*hc));
    if (e == cudaSuccess)
        e = for_each_step([&](auto fn, int ch) { return raise_smem(fn, step_smem_bytes(sb_max, max_n, ch)); });
    if (e == cudaSuccess)
        e = for_each_gstep([&](auto fn, int g) { return raise_smem(fn, gstep_smem_bytes(g, sb_max, max_n)); });
    return e;
}

cudaError_t raise_kernel_smem(int sort_cap, int sb_max, int max_n)
{
    std::lock_guard<std::mutex> lk(g_attr_mu);
    cudaError_t e = raise_smem(k_select, select_smem_bytes(sort_cap));
    if (e == cudaSuccess) e = raise_smem(k_select_cl<2>, select_smem_bytes(sort_cap));
    if (e == cudaSuccess) e = raise_smem(k_select_cl<4>, select_smem_bytes(sort_cap));
    if (e == cudaSuccess)
        e = for_each_step([&](auto fn, int ch) { return raise_smem(fn, step_smem_bytes(sb_max, max_n, ch)); });
    if (e == cudaSuccess)
        e = for_each_gstep([&](auto fn, int g) { return raise_smem(fn, gstep_smem_bytes(g, sb_max, max_n)); });
    return e;
}

#ifndef BSJ_PDL
#define BSJ_PDL 1
#endif

// Launch with (pdl) or without programmatic stream serialization after the previous
// kernel on the stream.
template <typename... KArgs, typename... Args>
static cudaError_t launch_kernel(void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t stream,
                                 bool pdl, Args... args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute at[1];
    if (pdl && BSJ_PDL) {
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
    }
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

template <int CH>
static cudaError_t launch_step_ch(const StepArgs& a, int s, int grid, int nq_mask, cudaStream_t stream)
{
    const size_t sm = step_smem_bytes(a.sb_max, a.max_n, CH);
    const int block = kWarpsPerStepCta * 32;
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess && (nq_mask & 2)) e = launch_kernel(k_step<1, CH>, grid, block, sm, stream, s >= 0, a, s);
    if (e == cudaSuccess && (nq_mask & 4)) e = launch_kernel(k_step<2, CH>, grid, block, sm, stream, s >= 0, a, s);
    if (e == cudaSuccess && (nq_mask & 16)) e = launch_kernel(k_step<4, CH>, grid, block, sm, stream, s >= 0, a, s);
    return e;
}

cudaError_t launch_step(const StepArgs& a, int s, int grid, int nq_mask, cudaStream_t stream)
{
    if (a.group_step) {
        const int G = a.group_step <= 2 ? 4 : 8;
        if (a.chunk != kGStepWarps * (32 / G)) return cudaErrorInvalidValue;
        const size_t sm = gstep_smem_bytes(G, a.sb_max, a.max_n);
        const int block = kGStepWarps * 32;
        switch (a.group_step) {
        case 1: return launch_kernel(k_step_g<4, 1>, grid, block, sm, stream, s >= 0, a, s);
        case 2: return launch_kernel(k_step_g<4, 2>, grid, block, sm, stream, s >= 0, a, s);
        case 3: return launch_kernel(k_step_g<8, 1>, grid, block, sm, stream, s >= 0, a, s);
        case 4: return launch_kernel(k_step_g<8, 2>, grid, block, sm, stream, s >= 0, a, s);
        default: return cudaErrorInvalidValue;
        }
    }
    switch (a.chunk) {
    case 8: return launch_step_ch<8>(a, s, grid, nq_mask, stream);
    case 16: return launch_step_ch<16>(a, s, grid, nq_mask, stream);
    case 32: return launch_step_ch<32>(a, s, grid, nq_mask, stream);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_gather_v1(const StepArgs& a, int s, int grid, cudaStream_t stream)
{
    return launch_kernel(k_gather_v1, grid, kWarpsPerStepCta * 32, 0, stream, true, a, s);
}

cudaError_t launch_select(const StepArgs& a, int s, int sort_cap, cudaStream_t stream)
{
    const int nseg = a.seg_hi - a.seg_lo;
    if (a.select_cluster <= 1)
        return launch_kernel(k_select, nseg, kSelectThreads, select_smem_bytes(sort_cap), stream, true, a, s,
                             sort_cap);
    const int C = a.select_cluster;
    if (C != 2 && C != 4) return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(nseg * C));
    cfg.blockDim = dim3((unsigned)kSelectThreads);
    cfg.dynamicSmemBytes = select_smem_bytes(sort_cap);
    cfg.stream = stream;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (BSJ_PDL) {
        at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[1].val.programmaticStreamSerializationAllowed = 1;
        cfg.numAttrs = 2;
    }
    return C == 2 ? cudaLaunchKernelEx(&cfg, k_select_cl<2>, a, s, sort_cap)
                  : cudaLaunchKernelEx(&cfg, k_select_cl<4>, a, s, sort_cap);
}

cudaError_t launch_heap(const StepArgs& a, int s, const HeapCfg& hc, cudaStream_t stream)
{
    return launch_kernel(k_heap, a.seg_hi - a.seg_lo, kHeapThreads, heap_smem_bytes(hc), stream, true, a, s, hc);
}

// The 1000 possible noise quotients of the gpu solvers' score, (float)(h % 1000) / 1e9f
// (gpu/v1/solver.cu:127), with the IEEE round-to-nearest division the reference compiles to.
// and of BS-PMS's, (double)(rand() % 1000) / 1000000.0 (cpu/v1_pms/solver.cpp:52-53).
__global__ void k_noise_table(float* noise, double* dnoise)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < 1000) {
        noise[k] = __fdiv_rn(__uint2float_rn((unsigned)k), 1000000000.0f);
        if (dnoise) dnoise[k] = __ddiv_rn((double)k, 1000000.0);
    }
}

cudaError_t launch_noise_table(float* noise, double* dnoise, cudaStream_t stream)
{
    k_noise_table<<<4, 256, 0, stream>>>(noise, dnoise);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const StepArgs& a, cudaStream_t stream)
{
    k_finalize<<<(a.nseg + 127) / 128, 128, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace bsj
