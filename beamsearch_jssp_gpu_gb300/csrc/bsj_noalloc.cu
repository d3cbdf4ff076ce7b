// bsj_noalloc.cu -- a single-beam solve that allocates no memory.
//
// Who needs it: callers that must not allocate device memory themselves or through us --
// operator/plugin hosts whose device memory is owned and budgeted by the host framework
// (an enqueue callback may only use the buffers it is handed), and latency-critical
// serving loops where a cudaMalloc/cudaFree would implicitly synchronise the device or
// fail at an arbitrary moment.  bsj_solve and the plan API allocate per context/plan;
// this entry point instead works inside one fixed scratch array that is part of the
// library's device image.
//
// The scratch is a file-scope __device__ array of BSJ_NOALLOC_SCRATCH_BYTES (64 MiB).
// Every GPU that loads the library holds it until the process exits.  Host code cannot
// pass the array's name to a kernel (on the host it is only a stand-in symbol, not a
// device address), so the first call on each device, with that device current, looks up
// its device address with cudaGetSymbolAddress and caches it; make that first call
// before any stream capture.  All calls share the one array, which keeps the previous
// call's contents: each call re-initialises every field that must start at zero.  Calls
// whose work overlaps on the GPU (different streams or threads, same device) race on the
// array and must be serialised by the caller.
//
// The kernels are the library's ordinary level kernels (k_step, k_select, k_finalize);
// only the buffers they are handed differ.  The per-call initial values reach the scratch
// as kernel parameters, not as copies from host memory, so a call only enqueues work on
// its stream and returns.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "../../include/bsj.h"
#include "bsj_kernels.h"

using namespace bsj;

namespace {

constexpr size_t kScratchBytes = BSJ_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once per device).
cudaError_t scratch_address(void** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// (duration << 8) | machine per op; an invalid entry is replaced by machine 0 / duration 0
// (so no kernel indexes outside the instance) and flags the beam state.  Durations whose
// sum reaches 2^31-1 would wrap the int32 makespans, so then the whole table is zeroed
// and the state flagged the same way.
__global__ void k_noalloc_pack(const int32_t* machine, const int32_t* duration, int count, int m,
                               uint32_t* ops, SegState* st)
{
    __shared__ unsigned long long total;
    if (threadIdx.x == 0) total = 0;
    __syncthreads();
    bool bad = false;
    unsigned long long local = 0;
    for (int q = threadIdx.x; q < count; q += blockDim.x) {
        int mc = machine[q], du = duration[q];
        if (mc < 0 || mc >= m || du < 0 || du > kMaxDuration) {
            bad = true;
            mc = 0;
            du = 0;
        }
        local += (unsigned long long)du;
        ops[q] = ((uint32_t)du << 8) | (uint32_t)mc;
    }
    atomicAdd(&total, local);
    __syncthreads();
    const bool overflow = total >= 0x7FFFFFFFull;
    if (overflow)
        for (int q = threadIdx.x; q < count; q += blockDim.x) ops[q] = 0u;
    if (bad || (threadIdx.x == 0 && overflow)) atomicOr(&st->status, 4);
}

// Per-call initial values of the beam's descriptor, state, prefixes and bound, written
// from kernel parameters (no host buffer is read, so nothing waits for the host).
__global__ void k_noalloc_init(SegDesc d, SegState st, int32_t beam_width, int32_t nch, int32_t group,
                               SegDesc* d_seg, SegState* d_st, int32_t* prefix, int32_t* cprefix,
                               int32_t* d_group)
{
    if (threadIdx.x == 0) {
        *d_seg = d;
        *d_st = st;
        prefix[0] = 0;
        prefix[1] = beam_width;
        cprefix[0] = 0;
        cprefix[1] = nch;
        *d_group = group;
    }
}

// Result into the caller's buffer: [0] makespan (-1 if the instance was invalid, -2 if a
// device consistency check of the level kernels failed), [1] found, [2 .. 2+N) sequence
// (zeros unless [0] >= 0).
__global__ void k_noalloc_out(const SegState* st, const int32_t* seq, int N, int32_t* out)
{
    const int status = st->status;
    const bool invalid = (status & 4) != 0;
    const bool corrupt = (status & (kStatusBadLineage | kStatusBadSelect)) != 0;
    const bool ok = !invalid && !corrupt;
    for (int t = threadIdx.x; t < N; t += blockDim.x) out[2 + t] = ok ? seq[t] : 0;
    if (threadIdx.x == 0) {
        out[0] = invalid ? -1 : (corrupt ? -2 : st->makespan);
        out[1] = ok ? st->found : 0;
    }
}

}  // namespace

extern "C" bsj_status bsj_solve_noalloc(int32_t n, int32_t m, const int32_t* d_machine,
                                        const int32_t* d_duration, int32_t mode, int32_t beam_width,
                                        int32_t best_known, uint32_t seed, int32_t* d_out, void* stream)
{
    if (!d_machine || !d_duration || !d_out) return BSJ_ERR_INVALID;
    if (mode != BSJ_MODE_V2 && mode != BSJ_MODE_CLEAN) return BSJ_ERR_INVALID;
    if (n < 1 || m < 1 || n > BSJ_MAX_JOBS || m > BSJ_MAX_MACHINES || (int64_t)n * m > BSJ_MAX_OPS)
        return BSJ_ERR_LIMIT;
    if (beam_width < 1 || beam_width > BSJ_MAX_BEAM) return BSJ_ERR_LIMIT;

    // one beam laid out exactly as a plan would lay it out
    SegDesc d{};
    d.n = n; d.m = m; d.N = n * m; d.K = beam_width;
    d.mode = mode; d.seed = seed;
    d.off_jr = 4 * m;
    d.off_rd = d.off_jr + 4 * n;
    d.off_nx = d.off_rd + n;
    d.off_hdr = (int)align_up((size_t)(d.off_nx + n), 4);
    d.sbytes = (int)align_up((size_t)d.off_hdr + 16, 16);
    d.words = (n + 31) / 32;
    d.auxbytes = 16;
    d.group = 0;
    d.op_off = 0;
    d.nq = nq_class(n);
    d.kcnt_off = 0;
    const int nch = (beam_width + kDefaultChunk - 1) / kDefaultChunk;
    const size_t K = (size_t)beam_width, N = (size_t)d.N;
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + bytes, 256); return at; };
    const size_t o_seg = take(sizeof(SegDesc));
    const size_t o_state = take(sizeof(SegState));
    const size_t o_prefix = take(2 * sizeof(int32_t));
    const size_t o_cprefix = take(2 * sizeof(int32_t));
    const size_t o_kcnt = take((size_t)nch * sizeof(int32_t));
    const size_t o_kmm = take((size_t)nch * sizeof(uint2));
    const size_t o_group = take(sizeof(int32_t));
    const size_t o_ops = take(N * sizeof(uint32_t));
    const size_t o_beam = take(2 * align_up(K * d.sbytes, 256));
    const size_t o_keys = take((size_t)nch * kDefaultChunk * n * 8);
    const size_t o_sel = take(K * 4);
    const size_t o_mask = take(K * d.words * 4);
    const size_t o_hist = take(N * K * 4);
    const size_t o_seq = take(N * 4);
    const size_t o_pos = take(2 * align_up(K * n, 256));
    const size_t o_noise = take(1000 * sizeof(float));
    if (o > kScratchBytes) return BSJ_ERR_LIMIT;  // beam_width x n*m too large for the scratch
    d.beam_off[0] = 0;
    d.beam_off[1] = (int64_t)align_up(K * d.sbytes, 256);
    d.key_off = d.sel_off = d.mask_off = d.hist_off = d.aux_off = d.seq_off = d.slot_off = 0;
    d.pos_off[0] = 0;
    d.pos_off[1] = (int64_t)align_up(K * n, 256);

    void* base_v = nullptr;
    if (scratch_address(&base_v) != cudaSuccess) return BSJ_ERR_CUDA;
    uint8_t* base = static_cast<uint8_t*>(base_v);
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    SegState st{};
    st.P = 1;
    st.bound = best_known;
    st.best = ~0ull;
    st.best_cmax = kSentinel;

    StepArgs a{};
    a.segs = reinterpret_cast<const SegDesc*>(base + o_seg);
    a.st = reinterpret_cast<SegState*>(base + o_state);
    a.rank_prefix = reinterpret_cast<const int32_t*>(base + o_prefix);
    a.nseg = 1;
    a.total_ranks = beam_width;
    a.seg_lo = 0;
    a.seg_hi = 1;
    a.chunk_lo = 0;
    a.chunk_hi = nch;
    a.rank_lo = 0;
    a.rank_hi = beam_width;
    a.chunk = kDefaultChunk;
    a.chunk_prefix = reinterpret_cast<const int32_t*>(base + o_cprefix);
    a.total_chunks = nch;
    a.kcnt = reinterpret_cast<int32_t*>(base + o_kcnt);
    a.kmm = reinterpret_cast<uint2*>(base + o_kmm);
    a.sb_max = d.sbytes;
    a.max_n = n;
    a.beam_pool = base + o_beam;
    a.slot_pool = nullptr;
    a.keys = reinterpret_cast<unsigned long long*>(base + o_keys);
    a.sel = reinterpret_cast<uint32_t*>(base + o_sel);
    a.masks = reinterpret_cast<uint32_t*>(base + o_mask);
    a.hist = reinterpret_cast<uint32_t*>(base + o_hist);
    a.aux_pool = nullptr;
    a.ops = reinterpret_cast<const uint32_t*>(base + o_ops);
    a.group_best = reinterpret_cast<int32_t*>(base + o_group);
    a.seq_pool = reinterpret_cast<int32_t*>(base + o_seq);
    a.pos_pool = base + o_pos;
    a.noise = reinterpret_cast<const float*>(base + o_noise);

    int sort_cap = 1;
    while (sort_cap < beam_width) sort_cap <<= 1;
    int sms = 0, dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return BSJ_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return BSJ_ERR_CUDA;
    if (raise_kernel_smem(sort_cap, d.sbytes, n) != cudaSuccess) return BSJ_ERR_CUDA;
    const int grid = std::max(1, nch);
    const int nq_mask = 1 << d.nq;

    // everything that must start at zero or at its initial value is rewritten here
    k_noalloc_init<<<1, 32, 0, s>>>(d, st, beam_width, nch, best_known,
                                    reinterpret_cast<SegDesc*>(base + o_seg),
                                    reinterpret_cast<SegState*>(base + o_state),
                                    reinterpret_cast<int32_t*>(base + o_prefix),
                                    reinterpret_cast<int32_t*>(base + o_cprefix),
                                    reinterpret_cast<int32_t*>(base + o_group));
    if (cudaGetLastError() != cudaSuccess) return BSJ_ERR_CUDA;
    if (cudaMemsetAsync(base + o_beam, 0, 2 * align_up(K * d.sbytes, 256), s) != cudaSuccess) return BSJ_ERR_CUDA;
    k_noalloc_pack<<<1, 256, 0, s>>>(d_machine, d_duration, d.N, m, reinterpret_cast<uint32_t*>(base + o_ops),
                                     reinterpret_cast<SegState*>(base + o_state));
    if (cudaGetLastError() != cudaSuccess) return BSJ_ERR_CUDA;
    if (launch_noise_table(reinterpret_cast<float*>(base + o_noise), nullptr, s) != cudaSuccess) return BSJ_ERR_CUDA;
    if (launch_step(a, -1, grid, nq_mask, s) != cudaSuccess) return BSJ_ERR_CUDA;
    for (int lv = 0; lv < d.N; lv++) {
        if (launch_select(a, lv, sort_cap, s) != cudaSuccess) return BSJ_ERR_CUDA;
        if (lv < d.N - 1 && launch_step(a, lv, grid, nq_mask, s) != cudaSuccess) return BSJ_ERR_CUDA;
    }
    if (launch_finalize(a, s) != cudaSuccess) return BSJ_ERR_CUDA;
    k_noalloc_out<<<1, 256, 0, s>>>(reinterpret_cast<const SegState*>(base + o_state),
                                    reinterpret_cast<const int32_t*>(base + o_seq), d.N, d_out);
    if (cudaGetLastError() != cudaSuccess) return BSJ_ERR_CUDA;
    return BSJ_OK;
}
