// bsj_engine.cu -- host engine and the C ABI (include/bsj.h).
//
// A plan is a set of beams (independent seeds and/or instances of uneven size, any mix
// of modes) laid out in one device allocation.  Running a plan enqueues every search level:
//
//   k_step(-1)                                   roots + level-0 expansion
//   for s = 0 .. maxN-1:
//       k_select(s) / k_heap(s)                  top-K per beam (gpu modes / ICH, PMS)
//       k_gather_v1(s)                           v1 beams only
//       k_step(s)            (s < maxN-1)        materialise level s+1, expand it
//   k_finalize                                   makespans + schedules
//
// replacing the reference's per-call host loop of three launches per level with device
// memory allocated once per call (gpu/v1/solver.cu:178-298, gpu/v2_twophases/solver.cu:
// 256-386).  The whole sequence is captured once into a CUDA graph and replayed.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bsj.h"
#include "bsj_kernels.h"

using namespace bsj;

#ifndef BSJ_MAX_BRANCHES
#define BSJ_MAX_BRANCHES 8
#endif
constexpr int kMaxBranches = BSJ_MAX_BRANCHES;  // beam groups run as concurrent graph branches

struct bsj_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t branch[kMaxBranches] = {};  // independent beam groups run on these
    std::string err;
    int sm_count = 0;
    int max_smem_optin = 0;
    // plans of recent batch shapes (most recent last), reused with new data
    std::vector<std::pair<std::string, bsj_plan*>> cache;
    uint64_t hits = 0;
    bool autotune = false;  // tune each new batch shape on its first bsj_solve_batch
};

struct bsj_plan {
    bsj_context* ctx = nullptr;
    int nseg = 0, ninst = 0, ngroups = 0;
    int maxN = 0;
    int total_ranks = 0;
    int nq_mask = 0;
    // k_step form: variant 0 runs every group with the step variant the default rule gives
    // it (Group::rule_var), variant 1 + v every group with step variant v (kStepVariant*:
    // warp per survivor with 8/16/32 per CTA, or thread per survivor).  Set by the
    // default, a tuning-table hit, bsj_plan_autotune or bsj_plan_set_chunk.
    int variant = 0;
    int select_force = 0;   // kSel* route flags of k_select (bsj_plan_set_select_route)
    int total_chunks[kNumChunkSizes] = {};
    int gather_grid = 1;
    int sort_cap = 0;
    HeapCfg heap{0, 1, 16, 1};   // k_heap configuration (ICH/PMS beams)
    bool has_v1 = false, has_zero = false, has_gpu = false, has_compat = false;
    // beam groups: contiguous beam ranges run as independent graph branches, so one
    // group's select overlaps the others' expansion
    struct Group {
        StepArgs args;   // chunk fields are filled per chunk size by group_args()
        int maxN = 0, nq_mask = 0, gather_grid = 1;
        int rule_var = 1;  // step variant (index into kStepVariant*) of the default rule
        int step_grid[kNumStepVariants] = {};
        bool has_v1 = false, has_gpu = false, has_compat = false;
        bool group_ok = false;   // every beam gpu-v2 / clean: the lane-group k_step applies
        int kmax_gpu = 0;        // widest gpu-mode beam (the cluster select is launched from
                                 // kSelectClusterMinK on)
        int64_t knmax_gpu = 0;   // largest K * n of its gpu-mode beams (4 CTAs per beam from
                                 // kSelectClusterWideKN on)
    };
    std::vector<Group> groups;
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[kMaxBranches] = {};
    std::vector<SegDesc> segs;
    std::vector<SegState> init;
    std::vector<int32_t> prefix;
    std::vector<int32_t> cprefix[kNumChunkSizes];  // per chunk size: prefix sums of ceil(K/chunk)
    std::vector<int32_t> group_init;
    std::vector<int32_t> seg_group;
    // segment i holds the caller's beam perm[i]: beams are laid out longest search first so
    // that the graph branches (contiguous segment ranges) group searches of similar length
    std::vector<int32_t> perm;
    std::string shape;  // shape_key() of the batch the plan was built for
    // device
    void* mem = nullptr;
    size_t mem_bytes = 0;
    SegDesc* d_segs = nullptr;
    SegState* d_state = nullptr;
    SegState* d_state_init = nullptr;
    int32_t* d_prefix = nullptr;
    int32_t* d_cprefix = nullptr;   // kNumChunkSizes arrays of nseg+1
    int32_t* d_group = nullptr;
    int32_t* d_group_init = nullptr;
    size_t beam_bytes = 0, slot_bytes = 0;
    StepArgs args{};
    // graphs per chunk variant: [0] plain, [1] with timing events recorded around each
    // launch; [2], [3] the same with the cluster select switched off
    cudaGraphExec_t graph[kNumStepVariants + 1][4] = {};
    bool select_cluster = true;   // bsj_plan_set_select_cluster: the cluster select where the rule picks it
    bool cluster_matters = false; // some beam group is wide enough for the rule to pick it
    int cluster_beams = 0;        // gpu-mode beams of K >= kSelectClusterMinK (their selects run at once)
    // timing
    bool timing = false;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> events;
    size_t events_used = 0;
    int64_t launches = 0;
    cudaStream_t last_stream = nullptr;
};

namespace {

constexpr const char* kVersion = "bsj-gb300 0.1.0 (sm_103a)";

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

bsj_status fail(bsj_context* ctx, bsj_status s, const std::string& msg)
{
    if (ctx) ctx->err = msg;
    return s;
}

bsj_status cuda_fail(bsj_context* ctx, cudaError_t e, const char* what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (ctx) ctx->err = m;
    return (e == cudaErrorMemoryAllocation) ? BSJ_ERR_NOMEM : BSJ_ERR_CUDA;
}

#define BSJ_CUDA(ctx, call)                                    \
    do {                                                       \
        cudaError_t _e = (call);                               \
        if (_e != cudaSuccess) return cuda_fail(ctx, _e, #call); \
    } while (0)

// glibc srand()/rand() state (published algorithm of glibc random_r.c, TYPE_3): r[0] =
// seed (1 if 0), r[i] = 16807*r[i-1] mod (2^31-1) for i < 31 via Schrage's method,
// r[i] = r[i-31] for 31..33, r[i] = r[i-31] + r[i-3] afterwards; outputs start at r[344].
// ring[i mod 34] holds r[i] for the last 34 positions.
void glibc_rand_state(uint32_t seed, uint32_t ring[34], uint32_t* next_index)
{
    std::vector<uint32_t> r(344);
    int64_t word = (int32_t)(seed == 0 ? 1u : seed);
    r[0] = (uint32_t)word;
    for (int k = 1; k < 31; k++) {
        int64_t hi = word / 127773, lo = word % 127773;
        word = 16807 * lo - 2836 * hi;
        if (word < 0) word += 2147483647;
        r[k] = (uint32_t)word;
    }
    for (int k = 31; k < 34; k++) r[k] = r[k - 31];
    for (int k = 34; k < 344; k++) r[k] = r[k - 31] + r[k - 3];
    for (int k = 310; k < 344; k++) ring[k % 34] = r[k];
    *next_index = 34 + 344 % 34;  // position 344, kept in [34, 68) like the device stream
}

bsj_status validate_instance(bsj_context* ctx, const bsj_instance& in)
{
    if (in.n < 1 || in.m < 1 || !in.machine || !in.duration)
        return fail(ctx, BSJ_ERR_INVALID, "instance: n, m must be >= 1 and arrays non-NULL");
    if (in.n > BSJ_MAX_JOBS || in.m > BSJ_MAX_MACHINES || (int64_t)in.n * in.m > BSJ_MAX_OPS)
        return fail(ctx, BSJ_ERR_LIMIT, "instance: n <= 128, m <= 64, n*m <= 8192 supported");
    int64_t total = 0;
    for (int64_t q = 0; q < (int64_t)in.n * in.m; q++) {
        if (in.machine[q] < 0 || in.machine[q] >= in.m)
            return fail(ctx, BSJ_ERR_INVALID, "instance: machine id outside [0, m)");
        if (in.duration[q] < 0 || in.duration[q] > BSJ_MAX_DURATION)
            return fail(ctx, BSJ_ERR_LIMIT, "instance: durations must lie in [0, 2^24)");
        total += in.duration[q];
    }
    if (total >= (int64_t)INT32_MAX)
        return fail(ctx, BSJ_ERR_LIMIT, "instance: total duration must fit int32");
    return BSJ_OK;
}

std::string shape_key(int ninst, const bsj_instance* insts, int nbeams, const bsj_beam* beams);

// ---- k_step chunk size: tuning table and default rule ----
// The table maps (device, plan shape) to the chunk size bsj_plan_autotune measured fastest;
// it is shared by every context and server of the process, so a shape tuned once (e.g. by
// a warm-up batch) is reused by later plans of that shape on any context.
std::mutex g_tune_mu;
std::vector<std::pair<std::string, int>> g_tuned;  // most recent last
constexpr size_t kTuneTable = 1024;

std::string tune_key(const bsj_context* ctx, const std::string& shape)
{
    return std::to_string(ctx->device) + "#" + shape;
}

int tuned_chunk(const bsj_context* ctx, const std::string& shape)
{
    const std::string k = tune_key(ctx, shape);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (const auto& e : g_tuned)
        if (e.first == k) return e.second;
    return -1;
}

void remember_chunk(const bsj_context* ctx, const std::string& shape, int v)
{
    const std::string k = tune_key(ctx, shape);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (auto& e : g_tuned)
        if (e.first == k) { e.second = v; return; }
    if (g_tuned.size() >= kTuneTable) g_tuned.erase(g_tuned.begin());
    g_tuned.push_back({k, v});
}

int chunk_var_of(int chunk)
{
    for (int v = 0; v < kNumChunkSizes; v++)
        if (kChunkSizes[v] == chunk) return v;
    return -1;
}

// Step variant (index into kStepVariant*) of a public chunk code; -1 if none.
int step_var_of_code(int code)
{
    for (int v = 0; v < kNumStepVariants; v++)
        if (kStepVariantCode[v] == code) return v;
    return -1;
}

// Default rule for one beam group: `ranks` = survivors per level of the whole plan (all
// groups run at once), `nq` = ceil(n/32) class holding most of the group's survivors,
// `granks` = the group's own survivors per level, `group_ok` = every beam of the group is
// gpu-v2 / clean (the lane-group forms apply).  Measured on GB300 (bench.py --chunk-sweep,
// gpu-v2, 18 shapes from 10x5 K=256 to 100x20 8x4096):
//  - lane-group forms: 8 lanes per survivor (16 per CTA) wins every shape with more than
//    2 048 survivors per level and n <= 64 (8 beams x 4 096 at 50x20: 32.3 vs 37.0 ms for
//    the best warp form; 20x15 8x4 096: 8.0 vs 10.6 ms), except one group of more than
//    8 192, where 4 lanes with a bulk copy win (K=16 384 at 20x15: 33.4 vs 35.8 ms); for
//    n > 64 from 4 096 survivors on, 4 lanes with a bulk copy (100x20 8x4 096: 112.2 vs
//    120.4 ms); narrower levels keep the 8-survivor warp form (single beams of K <= 1 024:
//    3-15 % faster than the group forms);
//  - other groups (v1, ICH/PMS): up to 8 192 survivors per level 8 per CTA, except n > 64
//    at 4 096 and more, where 32 wins; wider plans 16 per CTA, and 32 where the group alone
//    holds more than 8 192 or n > 64.
int rule_chunk_var(int64_t ranks, int nq, int64_t granks, bool group_ok, int kmax)
{
    if (group_ok) {
        // n > 64: the 8-lane bulk form for levels of K >= 2048 survivors (GB300, ms per search:
        // 100x20 K=4096 1 beam 63.3 -> 53.7, K=2048 8 beams 68.4 -> 57.5, 80x15 K=4096 8 beams
        // 42.0 -> 37.2 against the 4-lane form), 8 survivors per warp-form CTA below (100x20
        // K=1024 8 beams: 45.1 against 49.5 for the 8-lane form)
        if (nq == 4) return kmax >= 2048 ? step_var_of_code(4) : chunk_var_of(8);
        if (ranks <= 2048) return chunk_var_of(8);
        return granks > 8192 ? step_var_of_code(2) : step_var_of_code(3);
    }
    if (ranks <= 8192) return chunk_var_of((nq == 4 && ranks >= 4096) ? 32 : 8);
    return chunk_var_of((nq == 4 || granks > 8192) ? 32 : 16);
}

// With `bytes_only` non-null, computes the plan's device footprint into it and allocates
// nothing (*out is left untouched).
bsj_status plan_build(bsj_context* ctx, int ninst, const bsj_instance* insts, int nbeams,
                      const bsj_beam* beams, bsj_plan** out, size_t* bytes_only = nullptr)
{
    if (!ctx || (!out && !bytes_only) || ninst < 1 || nbeams < 1 || !insts || !beams)
        return fail(ctx, BSJ_ERR_INVALID, "plan: null argument or empty batch");
    for (int i = 0; i < ninst; i++) {
        bsj_status s = validate_instance(ctx, insts[i]);
        if (s != BSJ_OK) return s;
    }
    bsj_plan* p = new bsj_plan();
    p->ctx = ctx;
    p->nseg = nbeams;
    p->ninst = ninst;
    p->shape = shape_key(ninst, insts, nbeams, beams);

    // op tables: (duration << 8) | machine
    std::vector<uint32_t> ops;
    std::vector<int32_t> inst_off(ninst);
    for (int i = 0; i < ninst; i++) {
        inst_off[i] = (int32_t)ops.size();
        for (int64_t q = 0; q < (int64_t)insts[i].n * insts[i].m; q++)
            ops.push_back(((uint32_t)insts[i].duration[q] << 8) | (uint32_t)insts[i].machine[q]);
    }

    // bound groups
    std::vector<int> gid(nbeams);
    {
        std::vector<int> user_groups;
        int next = 0;
        std::vector<std::pair<int, int>> map;
        for (int b = 0; b < nbeams; b++) {
            int g = beams[b].bound_group;
            if (g < 0) { gid[b] = next++; continue; }
            auto it = std::find_if(map.begin(), map.end(), [&](const std::pair<int, int>& x) { return x.first == g; });
            if (it == map.end()) { map.push_back({g, next}); gid[b] = next++; }
            else gid[b] = it->second;
        }
        p->ngroups = next;
        p->group_init.assign(next, INT32_MAX);
    }

    // segment order: levels (n*m) descending, then the caller's order
    p->perm.resize(nbeams);
    for (int b = 0; b < nbeams; b++) p->perm[b] = b;
    auto levels_of = [&](int b) {
        const int i = beams[b].instance;
        return (i >= 0 && i < ninst) ? insts[i].n * insts[i].m : 0;
    };
    std::stable_sort(p->perm.begin(), p->perm.end(), [&](int x, int y) { return levels_of(x) > levels_of(y); });

    // per-beam layout
    size_t off_beam = 0, off_slot = 0, off_keys = 0, off_sel = 0, off_mask = 0, off_hist = 0, off_kcnt = 0,
           off_aux = 0, off_seq = 0, off_pos = 0;
    int sb_max = 16, max_n = 1;
    p->prefix.push_back(0);
    for (int v = 0; v < kNumChunkSizes; v++) p->cprefix[v].push_back(0);
    for (int si = 0; si < nbeams; si++) {
        const int b = p->perm[si];
        const bsj_beam& bm = beams[b];
        if (bm.instance < 0 || bm.instance >= ninst) { delete p; return fail(ctx, BSJ_ERR_INVALID, "beam: instance index out of range"); }
        if (bm.mode < BSJ_MODE_V1 || bm.mode > BSJ_MODE_PMS) { delete p; return fail(ctx, BSJ_ERR_INVALID, "beam: unknown mode"); }
        if (bm.beam_width < 1 || bm.beam_width > BSJ_MAX_BEAM) { delete p; return fail(ctx, BSJ_ERR_LIMIT, "beam: beam_width must lie in [1, 16384]"); }
        const bsj_instance& in = insts[bm.instance];
        SegDesc d{};
        d.n = in.n; d.m = in.m; d.N = in.n * in.m; d.K = bm.beam_width;
        d.mode = bm.mode; d.seed = bm.seed;
        d.off_jr = 4 * d.m;
        d.off_rd = d.off_jr + 4 * d.n;
        d.off_nx = d.off_rd + d.n;
        d.off_hdr = (int)align_up((size_t)(d.off_nx + d.n), 4);
        d.sbytes = (int)align_up((size_t)d.off_hdr + 16, 16);
        d.words = (d.n + 31) / 32;
        d.auxbytes = (int)align_up((size_t)(4 + 6 * d.n), 16);
        d.group = gid[b];
        d.op_off = inst_off[bm.instance];
        d.nq = nq_class(d.n);
        p->nq_mask |= 1 << d.nq;
        // per-chunk key counts for the smallest chunk size (the most chunks), key regions
        // for the largest (the most padding)
        d.kcnt_off = (int32_t)off_kcnt;
        off_kcnt += (d.K + kMinChunk - 1) / kMinChunk;
        const size_t K = (size_t)d.K, n = (size_t)d.n, N = (size_t)d.N;
        const bool gpu = d.mode <= BSJ_MODE_CLEAN;
        const int nbuf = (d.mode == BSJ_MODE_V1) ? 1 : 2;
        d.beam_off[0] = (int64_t)off_beam;
        d.beam_off[1] = (int64_t)(off_beam + (nbuf == 2 ? align_up(K * d.sbytes, 256) : 0));
        off_beam += nbuf * align_up(K * d.sbytes, 256);
        d.slot_off = (int64_t)off_slot;
        if (d.mode == BSJ_MODE_V1) off_slot += align_up(K * n * d.sbytes, 256);
        d.key_off = (int64_t)off_keys;
        if (gpu) off_keys += align_up((size_t)((d.K + kMaxChunk - 1) / kMaxChunk) * kMaxChunk * n, 32);
        d.sel_off = (int64_t)off_sel;
        off_sel += align_up(K, 64);
        d.mask_off = (int64_t)off_mask;
        if (gpu) off_mask += align_up(K * d.words, 64);
        d.hist_off = (int64_t)off_hist;
        off_hist += align_up(N * K, 64);
        d.aux_off = (int64_t)off_aux;
        if (!gpu) off_aux += align_up(K * d.auxbytes, 256);
        d.seq_off = (int64_t)off_seq;
        off_seq += align_up(N, 64);
        d.pos_off[0] = d.pos_off[1] = (int64_t)off_pos;
        if (d.mode == BSJ_MODE_V2 || d.mode == BSJ_MODE_CLEAN) {
            d.pos_off[1] = (int64_t)(off_pos + align_up(K * n, 256));
            off_pos += 2 * align_up(K * n, 256);
        }
        p->segs.push_back(d);
        p->prefix.push_back(p->prefix.back() + d.K);
        for (int v = 0; v < kNumChunkSizes; v++)
            p->cprefix[v].push_back(p->cprefix[v].back() + (d.K + kChunkSizes[v] - 1) / kChunkSizes[v]);
        sb_max = std::max(sb_max, d.sbytes);
        max_n = std::max(max_n, d.n);
        p->maxN = std::max(p->maxN, d.N);
        if (d.mode == BSJ_MODE_V1) p->has_v1 = true;
        if (d.mode == BSJ_MODE_V1 || d.mode == BSJ_MODE_V2) p->has_zero = true;
        if (gpu) { p->has_gpu = true; p->sort_cap = std::max(p->sort_cap, d.K); }
        else {
            p->has_compat = true;
            p->heap.kmax = std::max(p->heap.kmax, d.K);
            p->heap.ab = std::max(p->heap.ab, d.auxbytes);
            p->heap.nmax = std::max(p->heap.nmax, d.n);
        }

        SegState st{};
        st.P = 1;
        st.V = 0;
        st.bound = bm.best_known;
        st.best = ~0ull;
        st.best_cmax = kSentinel;
        if (!gpu) glibc_rand_state(bm.seed, st.rng, &st.rng_i);
        p->init.push_back(st);
        p->group_init[gid[b]] = std::min(p->group_init[gid[b]], bm.best_known);
        p->seg_group.push_back(gid[b]);
    }
    p->total_ranks = p->prefix.back();
    for (int v = 0; v < kNumChunkSizes; v++) p->total_chunks[v] = p->cprefix[v].back();
    if (p->has_gpu) {
        int sc = 1;
        while (sc < p->sort_cap) sc <<= 1;
        p->sort_cap = sc;
    }
    // ICH/PMS: the heap and the chunks of parents prepared ahead of it share the CTA's
    // shared memory; the chunk is as many parents as fit (at most kHeapMaxChunk)
    if (p->has_compat) {
        p->heap.chunk = heap_pick_chunk(p->heap, (size_t)ctx->max_smem_optin);
        if (p->heap.chunk < 1) { delete p; return fail(ctx, BSJ_ERR_LIMIT, "ICH/PMS beam too wide for shared memory"); }
    }
    if (p->has_gpu && select_smem_bytes(p->sort_cap) > (size_t)ctx->max_smem_optin) {
        delete p;
        return fail(ctx, BSJ_ERR_LIMIT, "beam too wide for the shared-memory select");
    }

    // device memory layout (one allocation)
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + bytes, 256); return at; };
    const size_t o_segs = take(sizeof(SegDesc) * nbeams);
    const size_t o_state = take(sizeof(SegState) * nbeams);
    const size_t o_state_init = take(sizeof(SegState) * nbeams);
    const size_t o_prefix = take(sizeof(int32_t) * (nbeams + 1));
    const size_t o_cprefix = take(sizeof(int32_t) * (nbeams + 1) * kNumChunkSizes);
    const size_t o_kcnt = take(sizeof(int32_t) * off_kcnt);
    const size_t o_kmm = take(sizeof(uint2) * off_kcnt);
    const size_t o_group = take(sizeof(int32_t) * p->ngroups);
    const size_t o_group_init = take(sizeof(int32_t) * p->ngroups);
    const size_t o_ops = take(sizeof(uint32_t) * ops.size());
    const size_t o_beam = take(off_beam);
    const size_t o_slot = take(off_slot);
    const size_t o_keys = take(8 * off_keys);
    const size_t o_sel = take(4 * off_sel);
    const size_t o_mask = take(4 * off_mask);
    const size_t o_hist = take(4 * off_hist);
    const size_t o_aux = take(off_aux);
    const size_t o_seq = take(4 * off_seq);
    const size_t o_pos = take(off_pos);
    const size_t o_noise = take(1000 * sizeof(float));
    const size_t o_dnoise = take(1000 * sizeof(double));
    p->mem_bytes = o;
    p->beam_bytes = off_beam;
    p->slot_bytes = off_slot;
    if (bytes_only) {
        *bytes_only = o;
        delete p;
        return BSJ_OK;
    }

    {
        cudaError_t e = cudaMalloc(&p->mem, o);
        if (e != cudaSuccess) { delete p; return cuda_fail(ctx, e, "cudaMalloc(plan)"); }
    }
    uint8_t* base = static_cast<uint8_t*>(p->mem);
    p->d_segs = reinterpret_cast<SegDesc*>(base + o_segs);
    p->d_state = reinterpret_cast<SegState*>(base + o_state);
    p->d_state_init = reinterpret_cast<SegState*>(base + o_state_init);
    p->d_prefix = reinterpret_cast<int32_t*>(base + o_prefix);
    p->d_cprefix = reinterpret_cast<int32_t*>(base + o_cprefix);
    p->d_group = reinterpret_cast<int32_t*>(base + o_group);
    p->d_group_init = reinterpret_cast<int32_t*>(base + o_group_init);

    StepArgs& a = p->args;
    a.segs = p->d_segs;
    a.st = p->d_state;
    a.rank_prefix = p->d_prefix;
    a.nseg = nbeams;
    a.total_ranks = p->total_ranks;
    a.seg_lo = 0;
    a.seg_hi = nbeams;
    a.rank_lo = 0;
    a.rank_hi = p->total_ranks;
    a.kcnt = reinterpret_cast<int32_t*>(base + o_kcnt);
    a.kmm = reinterpret_cast<uint2*>(base + o_kmm);
    a.sb_max = sb_max;
    a.max_n = max_n;
    a.beam_pool = base + o_beam;
    a.slot_pool = base + o_slot;
    a.keys = reinterpret_cast<unsigned long long*>(base + o_keys);
    a.sel = reinterpret_cast<uint32_t*>(base + o_sel);
    a.masks = reinterpret_cast<uint32_t*>(base + o_mask);
    a.hist = reinterpret_cast<uint32_t*>(base + o_hist);
    a.aux_pool = base + o_aux;
    a.ops = reinterpret_cast<const uint32_t*>(base + o_ops);
    a.group_best = p->d_group;
    a.seq_pool = reinterpret_cast<int32_t*>(base + o_seq);
    a.pos_pool = base + o_pos;
    a.noise = reinterpret_cast<const float*>(base + o_noise);
    a.dnoise = reinterpret_cast<const double*>(base + o_dnoise);

    // uploads (synchronous: the host vectors are pageable)
    cudaStream_t st = ctx->stream;
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->d_segs, p->segs.data(), sizeof(SegDesc) * nbeams, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->d_state_init, p->init.data(), sizeof(SegState) * nbeams, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->d_prefix, p->prefix.data(), sizeof(int32_t) * (nbeams + 1), cudaMemcpyHostToDevice, st);
    for (int v = 0; v < kNumChunkSizes && e == cudaSuccess; v++)
        e = cudaMemcpyAsync(p->d_cprefix + (size_t)v * (nbeams + 1), p->cprefix[v].data(), sizeof(int32_t) * (nbeams + 1),
                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->d_group_init, p->group_init.data(), sizeof(int32_t) * p->ngroups, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + o_ops, ops.data(), sizeof(uint32_t) * ops.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_noise_table(reinterpret_cast<float*>(base + o_noise),
                                                        reinterpret_cast<double*>(base + o_dnoise), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaFree(p->mem);
        delete p;
        return cuda_fail(ctx, e, "plan upload");
    }

    e = configure_kernels(std::max(p->sort_cap, 1), p->has_compat ? &p->heap : nullptr, sb_max, max_n);
    if (e != cudaSuccess) {
        cudaFree(p->mem);
        delete p;
        return cuda_fail(ctx, e, "configure kernels");
    }
    int want = (p->total_ranks + kWarpsPerStepCta - 1) / kWarpsPerStepCta;
    p->gather_grid = std::max(1, std::min(want, ctx->sm_count * 8));
    // beam groups, balanced by work (K * levels); BSJ_MAX_BEAM_GROUPS in the environment
    // lowers the number of concurrent groups (1 = all beams in lockstep, for measurements)
    {
        int gmax = kMaxBranches;
        if (const char* env = std::getenv("BSJ_MAX_BEAM_GROUPS")) {
            const int v = std::atoi(env);
            if (v >= 1 && v < gmax) gmax = v;
        }
        const int G = std::min(nbeams, gmax);
        double total = 0;
        for (int b = 0; b < nbeams; b++) total += (double)p->segs[b].K * p->segs[b].N;
        int lo = 0;
        double acc = 0;
        for (int g = 0; g < G && lo < nbeams; g++) {
            int hi = lo + 1;
            acc += (double)p->segs[lo].K * p->segs[lo].N;
            const double target = total * (g + 1) / G;
            while (hi < nbeams && (nbeams - hi) > (G - 1 - g) && acc + 0.5 * (double)p->segs[hi].K * p->segs[hi].N <= target) {
                acc += (double)p->segs[hi].K * p->segs[hi].N;
                hi++;
            }
            if (g == G - 1) {
                while (hi < nbeams) { acc += (double)p->segs[hi].K * p->segs[hi].N; hi++; }
            }
            bsj_plan::Group gr;
            gr.args = p->args;
            gr.args.seg_lo = lo;
            gr.args.seg_hi = hi;
            gr.args.rank_lo = p->prefix[lo];
            gr.args.rank_hi = p->prefix[hi];
            gr.group_ok = true;
            for (int b = lo; b < hi; b++) {
                const SegDesc& d = p->segs[b];
                gr.maxN = std::max(gr.maxN, d.N);
                gr.nq_mask |= 1 << d.nq;
                if (d.mode == BSJ_MODE_V1) gr.has_v1 = true;
                if (d.mode <= BSJ_MODE_CLEAN) {
                    gr.has_gpu = true;
                    if (d.K >= kSelectClusterMinK) p->cluster_beams++;
                    gr.kmax_gpu = std::max(gr.kmax_gpu, d.K);
                    gr.knmax_gpu = std::max(gr.knmax_gpu, (int64_t)d.K * d.n);
                } else {
                    gr.has_compat = true;
                }
                if (d.mode != BSJ_MODE_V2 && d.mode != BSJ_MODE_CLEAN) gr.group_ok = false;
            }
            // k_step: one CTA per chunk
            for (int v = 0; v < kNumStepVariants; v++) {
                const int ci = chunk_var_of(kStepVariantChunk[v]);
                int g = p->cprefix[ci][hi] - p->cprefix[ci][lo];
                gr.step_grid[v] = std::max(1, std::min(g, 65535));
            }
            const int wr = (p->prefix[hi] - p->prefix[lo] + kWarpsPerStepCta - 1) / kWarpsPerStepCta;
            gr.gather_grid = std::max(1, std::min(wr, ctx->sm_count * 8));
            if (gr.has_gpu && gr.kmax_gpu >= kSelectClusterMinK) p->cluster_matters = true;
            p->groups.push_back(gr);
            lo = hi;
        }
        // too many wide beams for even 2 CTAs each: the select form cannot differ
        if ((int64_t)p->cluster_beams * 2 > ctx->sm_count) p->cluster_matters = false;
        cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
        for (int g = 0; g < (int)p->groups.size(); g++) cudaEventCreateWithFlags(&p->join[g], cudaEventDisableTiming);
    }
    // chunk sizes: the default rule per group; the variant tuning found for this shape on
    // this device, else the rule
    for (auto& gr : p->groups) {
        int64_t per_nq[5] = {0, 0, 0, 0, 0};
        for (int b = gr.args.seg_lo; b < gr.args.seg_hi; b++) per_nq[p->segs[b].nq] += p->segs[b].K;
        const int nq = per_nq[4] > per_nq[2] && per_nq[4] > per_nq[1] ? 4 : (per_nq[2] > per_nq[1] ? 2 : 1);
        gr.rule_var = rule_chunk_var(p->total_ranks, nq, per_nq[1] + per_nq[2] + per_nq[4], gr.group_ok, gr.kmax_gpu);
    }
    {
        const int v = tuned_chunk(ctx, p->shape);
        p->variant = v >= 0 ? v : 0;
    }
    *out = p;
    return BSJ_OK;
}

// Step variant (index into kStepVariant*) group `gr` runs with under the plan's variant.
int group_var(const bsj_plan* p, const bsj_plan::Group& gr)
{
    return p->variant == 0 ? gr.rule_var : p->variant - 1;
}

// The launch arguments of group `gr` (whole plan: nullptr) for step variant v.
StepArgs group_args(const bsj_plan* p, const bsj_plan::Group* gr, int v)
{
    StepArgs a = gr ? gr->args : p->args;
    const int lo = gr ? a.seg_lo : 0, hi = gr ? a.seg_hi : p->nseg;
    const int ci = chunk_var_of(kStepVariantChunk[v]);
    a.chunk = kStepVariantChunk[v];
    a.group_step = (gr && gr->group_ok) ? kStepVariantGroup[v] : 0;
    a.select_force = p->select_force;
    {
        const int fz = p->select_force;
        const bool cl = (fz & kSelForceCluster) || (p->select_cluster && gr && gr->kmax_gpu >= kSelectClusterMinK);
        // 4 CTAs per beam for the widest levels, 2 otherwise, and no more CTAs per level than
        // the device has SMs: a plan running many wide beams at once (a batch) would
        // otherwise trade its throughput for latency it does not need
        int csize = (gr && gr->knmax_gpu >= kSelectClusterWideKN) ? 4 : 2;
        while (csize > 1 && (int64_t)p->cluster_beams * csize > p->ctx->sm_count) csize /= 2;
        if ((fz & kSelForceCluster) && csize < 2) csize = 2;
        a.select_cluster = (cl && !(fz & kSelNoCluster) && csize > 1) ? csize : 1;
    }
    a.chunk_prefix = p->d_cprefix + (size_t)ci * (p->nseg + 1);
    a.chunk_lo = p->cprefix[ci][lo];
    a.chunk_hi = p->cprefix[ci][hi];
    a.total_chunks = p->total_chunks[ci];
    return a;
}

cudaEvent_t* next_events(bsj_plan* p, int cls)
{
    if (p->events_used == p->events.size()) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        p->events.push_back({cls, {a, b}});
    }
    auto& ev = p->events[p->events_used++];
    ev.first = cls;
    return &ev.second.first;
}

// Enqueue one run of the plan on `s` (`capturing`: s is being captured into a graph, so
// timing events become event-record nodes of the graph).
cudaError_t enqueue_run(bsj_plan* p, cudaStream_t s, bool capturing)
{
    const StepArgs a = group_args(p, nullptr, chunk_var_of(kDefaultChunk));  // finalize: chunk unused
    cudaError_t e;
    p->launches = 0;
    p->events_used = 0;
    auto record = [&](cudaEvent_t ev) {
        return capturing ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal) : cudaEventRecord(ev, s);
    };
    auto timed = [&](int cls, auto&& fn) -> cudaError_t {
        if (!p->timing) { p->launches++; return fn(); }
        cudaEvent_t* ev = next_events(p, cls);
        cudaError_t r = record(ev[0]);
        if (r != cudaSuccess) return r;
        r = fn();
        if (r != cudaSuccess) return r;
        p->launches++;
        return record(ev[1]);
    };
    e = cudaMemcpyAsync(p->d_state, p->d_state_init, sizeof(SegState) * p->nseg, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(p->d_group, p->d_group_init, sizeof(int32_t) * p->ngroups, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    if (p->has_zero) {
        // v1 / v2 read never-written slots; the reference sees a fresh allocation (zeros)
        e = cudaMemsetAsync(a.beam_pool, 0, p->beam_bytes, s);
        if (e != cudaSuccess) return e;
        if (p->slot_bytes) e = cudaMemsetAsync(a.slot_pool, 0, p->slot_bytes, s);
        if (e != cudaSuccess) return e;
    }
    // one beam group's level loop on stream gs
    auto group_loop = [&](const bsj_plan::Group& gr, cudaStream_t gs) -> cudaError_t {
        auto rec = [&](cudaEvent_t ev) {
            return capturing ? cudaEventRecordWithFlags(ev, gs, cudaEventRecordExternal) : cudaEventRecord(ev, gs);
        };
        auto timed_g = [&](int cls, auto&& fn) -> cudaError_t {
            if (!p->timing) { p->launches++; return fn(); }
            cudaEvent_t* ev = next_events(p, cls);
            cudaError_t r = rec(ev[0]);
            if (r != cudaSuccess) return r;
            r = fn();
            if (r != cudaSuccess) return r;
            p->launches++;
            return rec(ev[1]);
        };
        const int cv = group_var(p, gr);
        const StepArgs ga = group_args(p, &gr, cv);
        const int step_grid = gr.step_grid[cv];
        cudaError_t r = timed_g(0, [&] { return launch_step(ga, -1, step_grid, gr.nq_mask, gs); });
        if (r != cudaSuccess) return r;
        for (int lv = 0; lv < gr.maxN; lv++) {
            if (gr.has_gpu) {
                r = timed_g(1, [&] { return launch_select(ga, lv, p->sort_cap, gs); });
                if (r != cudaSuccess) return r;
            }
            if (gr.has_compat) {
                r = timed_g(2, [&] { return launch_heap(ga, lv, p->heap, gs); });
                if (r != cudaSuccess) return r;
            }
            if (lv < gr.maxN - 1) {
                if (gr.has_v1) {
                    r = timed_g(3, [&] { return launch_gather_v1(ga, lv, gr.gather_grid, gs); });
                    if (r != cudaSuccess) return r;
                }
                r = timed_g(0, [&] { return launch_step(ga, lv, step_grid, gr.nq_mask, gs); });
                if (r != cudaSuccess) return r;
            }
        }
        return cudaSuccess;
    };
    if (p->groups.size() <= 1) {
        e = group_loop(p->groups[0], s);
        if (e != cudaSuccess) return e;
    } else {
        e = cudaEventRecord(p->fork, s);
        if (e != cudaSuccess) return e;
        for (size_t g = 0; g < p->groups.size(); g++) {
            cudaStream_t gs = p->ctx->branch[g];
            e = cudaStreamWaitEvent(gs, p->fork, 0);
            if (e != cudaSuccess) return e;
            e = group_loop(p->groups[g], gs);
            if (e != cudaSuccess) return e;
            e = cudaEventRecord(p->join[g], gs);
            if (e != cudaSuccess) return e;
            e = cudaStreamWaitEvent(s, p->join[g], 0);
            if (e != cudaSuccess) return e;
        }
    }
    return timed(4, [&] { return launch_finalize(a, s); });
}

constexpr size_t kPlanCache = 4;

// Everything that fixes a plan's layout and graph: sizes, modes, widths, bound groups.
std::string shape_key(int ninst, const bsj_instance* insts, int nbeams, const bsj_beam* beams)
{
    std::string k = std::to_string(ninst) + "|";
    for (int i = 0; i < ninst; i++) k += std::to_string(insts[i].n) + "x" + std::to_string(insts[i].m) + ",";
    k += "|";
    for (int b = 0; b < nbeams; b++)
        k += std::to_string(beams[b].mode) + ":" + std::to_string(beams[b].beam_width) + ":" +
             std::to_string(beams[b].instance) + ":" + std::to_string(beams[b].bound_group) + ",";
    return k;
}

// New instance data, seeds and bounds into a plan of the same shape.
bsj_status plan_refresh(bsj_plan* p, int ninst, const bsj_instance* insts, const bsj_beam* beams)
{
    bsj_context* ctx = p->ctx;
    for (int i = 0; i < ninst; i++) {
        bsj_status s = validate_instance(ctx, insts[i]);
        if (s != BSJ_OK) return s;
    }
    std::vector<uint32_t> ops;
    for (int i = 0; i < ninst; i++)
        for (int64_t q = 0; q < (int64_t)insts[i].n * insts[i].m; q++)
            ops.push_back(((uint32_t)insts[i].duration[q] << 8) | (uint32_t)insts[i].machine[q]);
    std::fill(p->group_init.begin(), p->group_init.end(), INT32_MAX);
    for (int si = 0; si < p->nseg; si++) {
        const bsj_beam& bm = beams[p->perm[si]];
        p->segs[si].seed = bm.seed;
        SegState st{};
        st.P = 1;
        st.bound = bm.best_known;
        st.best = ~0ull;
        st.best_cmax = kSentinel;
        if (bm.mode > BSJ_MODE_CLEAN) glibc_rand_state(bm.seed, st.rng, &st.rng_i);
        p->init[si] = st;
        const int g = p->seg_group[si];
        p->group_init[g] = std::min(p->group_init[g], bm.best_known);
    }
    cudaStream_t st = ctx->stream;
    cudaError_t e = cudaMemcpyAsync(p->d_segs, p->segs.data(), sizeof(SegDesc) * p->nseg, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->d_state_init, p->init.data(), sizeof(SegState) * p->nseg, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->d_group_init, p->group_init.data(), sizeof(int32_t) * p->ngroups, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(const_cast<uint32_t*>(p->args.ops), ops.data(), sizeof(uint32_t) * ops.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "plan refresh");
    return BSJ_OK;
}

// The rand() stream of an ICH/PMS beam, carried from one pass to the next the way the
// process-wide state runs on between the reference's successive calls
// (cpu/v1_pms/main.cpp:56,64).
struct RandCarry {
    uint32_t i;  // position of the next value, in [34, 68)
    uint32_t r[34];
};

// Start each ICH/PMS beam of the plan's next run from `in[b]` instead of its seed.
bsj_status plan_put_rand(bsj_plan* p, const RandCarry* in)
{
    for (int si = 0; si < p->nseg; si++) {
        if (p->segs[si].mode <= BSJ_MODE_CLEAN) continue;
        const RandCarry& c = in[p->perm[si]];
        p->init[si].rng_i = 34 + (c.i % 34);
        std::memcpy(p->init[si].rng, c.r, sizeof(c.r));
    }
    cudaStream_t st = p->ctx->stream;
    cudaError_t e = cudaMemcpyAsync(p->d_state_init, p->init.data(), sizeof(SegState) * p->nseg,
                                    cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? BSJ_OK : cuda_fail(p->ctx, e, "rand state upload");
}

// Where each ICH/PMS beam's stream stands after the last run (call after the results).
bsj_status plan_get_rand(bsj_plan* p, RandCarry* out)
{
    std::vector<SegState> st(p->nseg);
    cudaError_t e = cudaMemcpy(st.data(), p->d_state, sizeof(SegState) * p->nseg, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(p->ctx, e, "rand state read");
    for (int si = 0; si < p->nseg; si++) {
        RandCarry& c = out[p->perm[si]];
        c.i = st[si].rng_i;
        std::memcpy(c.r, st[si].rng, sizeof(c.r));
    }
    return BSJ_OK;
}

bsj_status solve_batch_impl(bsj_context* ctx, int num_instances, const bsj_instance* instances,
                            int num_beams, const bsj_beam* beams, bsj_result* results, void* stream,
                            const RandCarry* rand_in, RandCarry* rand_out);

}  // namespace

// =====================================================================================
// C ABI
// =====================================================================================
// The plan's graph for its current chunk variant, timing and selection form, captured on
// first use (on the context's stream; it replays on any stream).
static bsj_status plan_graph(bsj_plan* p, cudaGraphExec_t** out)
{
    bsj_context* ctx = p->ctx;
    const bool cluster = p->select_cluster || !p->cluster_matters;   // one graph when it cannot differ
    const int gi = (p->timing ? 1 : 0) + (cluster ? 0 : 2);
    cudaGraphExec_t& graph = p->graph[p->variant][gi];
    if (!graph) {
        cudaStream_t cap = ctx->stream;
        cudaGraph_t g = nullptr;
        BSJ_CUDA(ctx, cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = enqueue_run(p, cap, true);
        cudaError_t e2 = cudaStreamEndCapture(cap, &g);
        if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(ctx, e, "plan capture"); }
        if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { graph = nullptr; return cuda_fail(ctx, e, "cudaGraphInstantiate"); }
    }
    *out = &graph;
    return BSJ_OK;
}

// Captures the plan's (untimed) graphs of both selection forms without running them, so a
// server can switch forms per request without a capture on its path.
namespace bsj {
bsj_status plan_capture_forms(bsj_plan* p)
{
    if (!p) return BSJ_ERR_INVALID;
    cudaSetDevice(p->ctx->device);
    const bool keep_cluster = p->select_cluster, keep_timing = p->timing;
    p->timing = false;
    bsj_status st = BSJ_OK;
    for (int on = 1; on >= 0 && st == BSJ_OK; on--) {
        p->select_cluster = on != 0;
        cudaGraphExec_t* graph = nullptr;
        st = plan_graph(p, &graph);
        if (!p->cluster_matters) break;
    }
    p->select_cluster = keep_cluster;
    p->timing = keep_timing;
    return st;
}
}  // namespace bsj

extern "C" {

const char* bsj_version(void) { return kVersion; }

bsj_status bsj_device_count(int32_t* count)
{
    if (!count) return BSJ_ERR_INVALID;
    int c = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    *count = (e == cudaSuccess) ? c : 0;
    if (e != cudaSuccess) cudaGetLastError();
    return e == cudaSuccess ? BSJ_OK : BSJ_ERR_CUDA;
}

const char* bsj_status_string(bsj_status s)
{
    switch (s) {
    case BSJ_OK: return "ok";
    case BSJ_ERR_INVALID: return "invalid argument";
    case BSJ_ERR_LIMIT: return "size outside the supported limits";
    case BSJ_ERR_CUDA: return "CUDA error";
    case BSJ_ERR_NOMEM: return "out of memory";
    case BSJ_ERR_DEVICE: return "device-side consistency check failed";
    }
    return "unknown status";
}

bsj_status bsj_create(bsj_context** out, int device)
{
    if (!out) return BSJ_ERR_INVALID;
    *out = nullptr;
    bsj_context* ctx = new bsj_context();
    cudaError_t e;
    if (device < 0) {
        e = cudaGetDevice(&device);
        if (e != cudaSuccess) { bsj_status s = cuda_fail(ctx, e, "cudaGetDevice"); delete ctx; return s; }
    }
    e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    for (int g = 0; g < kMaxBranches && e == cudaSuccess; g++)
        e = cudaStreamCreateWithFlags(&ctx->branch[g], cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete ctx; return BSJ_ERR_CUDA; }
    ctx->device = device;
    *out = ctx;
    return BSJ_OK;
}

void bsj_destroy(bsj_context* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    for (auto& kv : ctx->cache) bsj_plan_destroy(kv.second);
    ctx->cache.clear();
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    for (cudaStream_t b : ctx->branch)
        if (b) cudaStreamDestroy(b);
    delete ctx;
}

const char* bsj_last_error(const bsj_context* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

bsj_status bsj_plan_create(bsj_context* ctx, int num_instances, const bsj_instance* instances,
                           int num_beams, const bsj_beam* beams, bsj_plan** out)
{
    if (!ctx) return BSJ_ERR_INVALID;
    cudaSetDevice(ctx->device);
    return plan_build(ctx, num_instances, instances, num_beams, beams, out);
}

bsj_status bsj_plan_estimate(bsj_context* ctx, int num_instances, const bsj_instance* instances,
                             int num_beams, const bsj_beam* beams, int64_t* device_bytes)
{
    if (!ctx || !device_bytes) return BSJ_ERR_INVALID;
    size_t bytes = 0;
    bsj_status s = plan_build(ctx, num_instances, instances, num_beams, beams, nullptr, &bytes);
    if (s == BSJ_OK) *device_bytes = (int64_t)bytes;
    return s;
}

int64_t bsj_plan_device_bytes(const bsj_plan* p) { return p ? (int64_t)p->mem_bytes : 0; }

bsj_status bsj_plan_update(bsj_plan* p, int num_instances, const bsj_instance* instances, int num_beams,
                           const bsj_beam* beams)
{
    if (!p || !instances || !beams || num_instances != p->ninst || num_beams != p->nseg) return BSJ_ERR_INVALID;
    if (p->shape != shape_key(num_instances, instances, num_beams, beams))
        return fail(p->ctx, BSJ_ERR_INVALID, "plan update: sizes, modes, widths or groups differ from the plan's");
    cudaSetDevice(p->ctx->device);
    return plan_refresh(p, num_instances, instances, beams);
}

bsj_status bsj_plan_run(bsj_plan* p, void* stream)
{
    if (!p) return BSJ_ERR_INVALID;
    bsj_context* ctx = p->ctx;
    cudaSetDevice(ctx->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    p->last_stream = s;
    cudaGraphExec_t* graph = nullptr;
    const bsj_status st = plan_graph(p, &graph);
    if (st != BSJ_OK) return st;
    BSJ_CUDA(ctx, cudaGraphLaunch(*graph, s));
    return BSJ_OK;
}

bsj_status bsj_plan_results(bsj_plan* p, bsj_result* results)
{
    if (!p || !results) return BSJ_ERR_INVALID;
    bsj_context* ctx = p->ctx;
    cudaSetDevice(ctx->device);
    cudaStream_t s = p->last_stream ? p->last_stream : ctx->stream;
    BSJ_CUDA(ctx, cudaStreamSynchronize(s));
    std::vector<SegState> st(p->nseg);
    std::vector<int32_t> grp(p->ngroups);
    BSJ_CUDA(ctx, cudaMemcpy(st.data(), p->d_state, sizeof(SegState) * p->nseg, cudaMemcpyDeviceToHost));
    BSJ_CUDA(ctx, cudaMemcpy(grp.data(), p->d_group, sizeof(int32_t) * p->ngroups, cudaMemcpyDeviceToHost));
    bsj_status status = BSJ_OK;
    for (int si = 0; si < p->nseg; si++) {
        const SegDesc& d = p->segs[si];
        const int b = p->perm[si];
        bsj_result& r = results[b];
        r.makespan = st[si].makespan;
        r.found = st[si].found;
        r.expanded = st[si].expanded;
        r.slots = st[si].slots;
        r.levels = st[si].levels;
        r.group_best = grp[p->seg_group[si]];
        if (r.sequence) {
            BSJ_CUDA(ctx, cudaMemcpy(r.sequence, p->args.seq_pool + d.seq_off, sizeof(int32_t) * d.N, cudaMemcpyDeviceToHost));
        }
        if (st[si].status != 0) {
            status = BSJ_ERR_DEVICE;
            ctx->err = "beam " + std::to_string(b) + ": device status " + std::to_string(st[si].status);
        }
    }
    return status;
}

void bsj_plan_destroy(bsj_plan* p)
{
    if (!p) return;
    cudaSetDevice(p->ctx->device);
    for (auto& gv : p->graph)
        for (cudaGraphExec_t g : gv)
            if (g) cudaGraphExecDestroy(g);
    if (p->fork) cudaEventDestroy(p->fork);
    for (cudaEvent_t ev : p->join)
        if (ev) cudaEventDestroy(ev);
    for (auto& ev : p->events) {
        cudaEventDestroy(ev.second.first);
        cudaEventDestroy(ev.second.second);
    }
    if (p->mem) cudaFree(p->mem);
    delete p;
}

int64_t bsj_plan_launches(const bsj_plan* p)
{
    if (!p) return 0;
    // fixed by the plan shape: per group 1 + maxN*(select? + heap?) + (maxN-1)*(gather_v1? + step
    // launches per NQ class); one finalize
    int64_t n = 1;
    for (const auto& gr : p->groups) {
        const int64_t per = (gr.has_gpu ? 1 : 0) + (gr.has_compat ? 1 : 0);
        const int64_t nq = __builtin_popcount((unsigned)gr.nq_mask);
        n += nq + (int64_t)gr.maxN * per + (int64_t)(gr.maxN - 1) * (nq + (gr.has_v1 ? 1 : 0));
    }
    return n;
}

bsj_status bsj_plan_stats(const bsj_plan* p, double* step_bytes, double* select_bytes, int64_t* expanded,
                          int64_t* materialized, int64_t* select_fallbacks)
{
    if (!p) return BSJ_ERR_INVALID;
    std::vector<SegState> st(p->nseg);
    cudaSetDevice(p->ctx->device);
    cudaError_t e = cudaMemcpy(st.data(), p->d_state, sizeof(SegState) * p->nseg, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return BSJ_ERR_CUDA;
    double sb = 0.0, selb = 0.0;
    int64_t ex = 0, mat = 0, fb = 0;
    for (int b = 0; b < p->nseg; b++) {
        const SegDesc& d = p->segs[b];
        sb += (double)st[b].materialized * (2.0 * d.sbytes + 8.0) + 8.0 * (double)st[b].expanded;
        selb += 8.0 * (double)st[b].expanded + 4.0 * (double)st[b].materialized;
        ex += st[b].expanded;
        mat += st[b].materialized;
        fb += st[b].select_fallbacks;
    }
    if (select_fallbacks) *select_fallbacks = fb;
    if (step_bytes) *step_bytes = sb;
    if (select_bytes) *select_bytes = selb;
    if (expanded) *expanded = ex;
    if (materialized) *materialized = mat;
    return BSJ_OK;
}

bsj_status bsj_plan_set_timing(bsj_plan* p, int enable)
{
    if (!p) return BSJ_ERR_INVALID;
    p->timing = enable != 0;
    return BSJ_OK;
}

bsj_status bsj_plan_kernel_ms(const bsj_plan* p, float* ms, int64_t* launches, int count)
{
    if (!p || !ms) return BSJ_ERR_INVALID;
    for (int i = 0; i < count; i++) { ms[i] = 0.f; if (launches) launches[i] = 0; }
    cudaSetDevice(p->ctx->device);
    for (size_t k = 0; k < p->events_used; k++) {
        const auto& ev = p->events[k];
        float t = 0.f;
        cudaError_t e = cudaEventSynchronize(ev.second.second);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, ev.second.first, ev.second.second);
        if (e != cudaSuccess) return BSJ_ERR_CUDA;
        if (ev.first < count) {
            ms[ev.first] += t;
            if (launches) launches[ev.first]++;
        }
    }
    return BSJ_OK;
}

bsj_status bsj_plan_set_chunk(bsj_plan* p, int32_t chunk)
{
    if (!p) return BSJ_ERR_INVALID;
    if (chunk == 0) { p->variant = 0; return BSJ_OK; }
    const int v = step_var_of_code(chunk);
    if (v >= 0) {
        p->variant = 1 + v;
        return BSJ_OK;
    }
    return fail(p->ctx, BSJ_ERR_INVALID,
                "chunk must be 0 (default rule), 8, 16, 32 (warp per survivor) or 1, 2, 3, 4 "
                "(lane group per survivor)");
}

static_assert(BSJ_SELECT_FORCE_LARGE == kSelForceLarge && BSJ_SELECT_NO_LARGE == kSelNoLarge &&
              BSJ_SELECT_NO_DIRECT == kSelNoDirect && BSJ_SELECT_RADIX == kSelForceRadix &&
              BSJ_SELECT_NO_DENSE == kSelNoDense && BSJ_SELECT_RANK_LSD == kSelRankLsd &&
              BSJ_SELECT_BITONIC == kSelBitonic && BSJ_SELECT_NO_CLUSTER == kSelNoCluster &&
              BSJ_SELECT_FORCE_CLUSTER == kSelForceCluster, "route flags of bsj.h and the kernels differ");
static_assert(BSJ_ROUTE_LARGE == kPathLarge && BSJ_ROUTE_DIRECT == kPathDirect && BSJ_ROUTE_BUCKET == kPathBucket &&
              BSJ_ROUTE_RADIX == kPathRadix && BSJ_ROUTE_DENSE == kPathDense &&
              BSJ_ROUTE_RANK_LSD == kPathRankLsd && BSJ_ROUTE_RAW_LSD == kPathRawLsd &&
              BSJ_ROUTE_BITONIC == kPathBitonic && BSJ_ROUTE_CLUSTER == kPathCluster, "route bits of bsj.h and the kernels differ");

bsj_status bsj_plan_set_select_route(bsj_plan* p, int32_t flags)
{
    if (!p) return BSJ_ERR_INVALID;
    if ((flags & ~kSelAll) != 0 || ((flags & kSelForceLarge) && (flags & kSelNoLarge)) ||
        ((flags & kSelForceCluster) && (flags & kSelNoCluster)))
        return fail(p->ctx, BSJ_ERR_INVALID, "unknown or contradictory select route flags");
    if (flags == p->select_force) return BSJ_OK;
    // the flags are a launch argument baked into the captured graphs: capture again
    cudaSetDevice(p->ctx->device);
    for (auto& gv : p->graph)
        for (cudaGraphExec_t& g : gv)
            if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    p->select_force = flags;
    return BSJ_OK;
}

bsj_status bsj_plan_set_select_cluster(bsj_plan* p, int32_t enable)
{
    if (!p) return BSJ_ERR_INVALID;
    p->select_cluster = enable != 0;   // each form's graph is captured once and kept
    return BSJ_OK;
}

bsj_status bsj_plan_select_routes(bsj_plan* p, uint32_t* routes)
{
    if (!p || !routes) return BSJ_ERR_INVALID;
    bsj_context* ctx = p->ctx;
    cudaSetDevice(ctx->device);
    BSJ_CUDA(ctx, cudaStreamSynchronize(p->last_stream ? p->last_stream : ctx->stream));
    std::vector<SegState> st(p->nseg);
    BSJ_CUDA(ctx, cudaMemcpy(st.data(), p->d_state, sizeof(SegState) * p->nseg, cudaMemcpyDeviceToHost));
    uint32_t r = 0;
    for (const SegState& x : st) r |= x.select_paths;
    *routes = r;
    return BSJ_OK;
}

int32_t bsj_plan_chunk(const bsj_plan* p) { return (p && p->variant > 0) ? kStepVariantCode[p->variant - 1] : 0; }

bsj_status bsj_plan_autotune(bsj_plan* p, void* stream, int32_t repeats, int32_t* chunk, float* ms)
{
    if (!p) return BSJ_ERR_INVALID;
    bsj_context* ctx = p->ctx;
    cudaSetDevice(ctx->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    if (repeats < 1) repeats = 1;
    // a uniform size that the rule already gives every group is not timed twice
    int rule_uniform = -1;
    for (const auto& gr : p->groups) {
        if (rule_uniform == -1) rule_uniform = gr.rule_var;
        else if (rule_uniform != gr.rule_var) rule_uniform = -2;
    }
    const bool timing = p->timing;
    p->timing = false;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    bsj_status st = BSJ_OK;
    cudaError_t e = cudaEventCreate(&ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
    if (e != cudaSuccess) st = cuda_fail(ctx, e, "autotune events");
    float best = 0.f;
    int bv = -1;
    for (int v = 0; v <= kNumStepVariants && st == BSJ_OK; v++) {
        if (ms) ms[v] = -1.f;
        if (v > 0 && v - 1 == rule_uniform) {
            if (ms) ms[v] = ms[0];
            continue;
        }
        p->variant = v;
        st = bsj_plan_run(p, s);  // captures this variant's graph; untimed warm-up
        if (st != BSJ_OK) break;
        e = cudaEventRecord(ev[0], s);
        for (int r = 0; r < repeats && st == BSJ_OK && e == cudaSuccess; r++) st = bsj_plan_run(p, s);
        if (st != BSJ_OK) break;
        if (e == cudaSuccess) e = cudaEventRecord(ev[1], s);
        if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
        float t = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, ev[0], ev[1]);
        if (e != cudaSuccess) { st = cuda_fail(ctx, e, "autotune timing"); break; }
        t /= (float)repeats;
        if (ms) ms[v] = t;
        if (bv < 0 || t < best) { best = t; bv = v; }
    }
    for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
    p->timing = timing;
    if (st != BSJ_OK) { p->variant = 0; return st; }
    p->variant = bv;
    remember_chunk(ctx, p->shape, bv);
    if (chunk) *chunk = bsj_plan_chunk(p);
    return BSJ_OK;
}

bsj_status bsj_set_autotune(bsj_context* ctx, int32_t enable)
{
    if (!ctx) return BSJ_ERR_INVALID;
    ctx->autotune = enable != 0;
    return BSJ_OK;
}

bsj_status bsj_solve_batch(bsj_context* ctx, int num_instances, const bsj_instance* instances,
                           int num_beams, const bsj_beam* beams, bsj_result* results, void* stream)
{
    return solve_batch_impl(ctx, num_instances, instances, num_beams, beams, results, stream, nullptr, nullptr);
}

}  // extern "C"

namespace {

bsj_status solve_batch_impl(bsj_context* ctx, int num_instances, const bsj_instance* instances,
                            int num_beams, const bsj_beam* beams, bsj_result* results, void* stream,
                            const RandCarry* rand_in, RandCarry* rand_out)
{
    if (!ctx || !results || !instances || !beams || num_instances < 1 || num_beams < 1) return BSJ_ERR_INVALID;
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    const std::string key = shape_key(num_instances, instances, num_beams, beams);
    for (size_t i = 0; i < ctx->cache.size(); i++) {
        if (ctx->cache[i].first != key) continue;
        // same shape as a recent call: new data into the existing plan, replay its graph
        bsj_plan* p = ctx->cache[i].second;
        std::rotate(ctx->cache.begin() + i, ctx->cache.begin() + i + 1, ctx->cache.end());
        bsj_status s = plan_refresh(p, num_instances, instances, beams);
        if (s == BSJ_OK && rand_in) s = plan_put_rand(p, rand_in);
        if (s != BSJ_OK) return s;
        ctx->hits++;
        p->timing = false;
        s = bsj_plan_run(p, st);
        if (s == BSJ_OK) s = bsj_plan_results(p, results);
        if (s == BSJ_OK && rand_out) s = plan_get_rand(p, rand_out);
        return s;
    }
    bsj_plan* p = nullptr;
    bsj_status s = plan_build(ctx, num_instances, instances, num_beams, beams, &p);
    if (s == BSJ_OK && rand_in) {
        s = plan_put_rand(p, rand_in);
        if (s != BSJ_OK) bsj_plan_destroy(p);
    }
    if (s != BSJ_OK) return s;
    if (ctx->autotune && tuned_chunk(ctx, key) < 0) {
        // tune the new shape; every candidate run computes the same results
        s = bsj_plan_autotune(p, st, 1, nullptr, nullptr);
        if (s != BSJ_OK) { bsj_plan_destroy(p); return s; }
        s = bsj_plan_run(p, st);
        if (s != BSJ_OK) { bsj_plan_destroy(p); return s; }
    } else {
        // first call of this shape: eager launches (capturing a graph pays off on reuse only)
        p->last_stream = st;
        cudaError_t e = enqueue_run(p, st, false);
        if (e != cudaSuccess) { bsj_plan_destroy(p); return cuda_fail(ctx, e, "solve"); }
    }
    s = bsj_plan_results(p, results);
    if (s == BSJ_OK && rand_out) s = plan_get_rand(p, rand_out);
    if (s != BSJ_OK) { bsj_plan_destroy(p); return s; }
    if (ctx->cache.size() >= kPlanCache) {
        bsj_plan_destroy(ctx->cache.front().second);
        ctx->cache.erase(ctx->cache.begin());
    }
    ctx->cache.push_back({key, p});
    return BSJ_OK;
}

}  // namespace

extern "C" {

bsj_status bsj_solve(bsj_context* ctx, const bsj_instance* inst, const bsj_beam* beam,
                     bsj_result* result, void* stream)
{
    if (!ctx || !inst || !beam || !result) return BSJ_ERR_INVALID;
    bsj_beam b = *beam;
    b.instance = 0;
    return bsj_solve_batch(ctx, 1, inst, 1, &b, result, stream);
}

bsj_status bsj_solve_iterations(bsj_context* ctx, const bsj_instance* inst, int mode, int beam_width,
                                int num_beams, int iterations, const uint32_t* seeds,
                                int32_t initial_bound, int32_t* best, int32_t* best_sequence,
                                int32_t* round_best, void* stream)
{
    if (!ctx || !inst || !seeds || num_beams < 1 || iterations < 1) return BSJ_ERR_INVALID;
    if (inst->n < 1 || inst->m < 1) return BSJ_ERR_INVALID;
    // ICH/PMS ranks srand() once and draw on from round to round (cpu/v1_pms/main.cpp:56-67)
    const bool carry = (mode == BSJ_MODE_ICH || mode == BSJ_MODE_PMS);
    std::vector<RandCarry> rng(carry ? num_beams : 0);
    for (int b = 0; b < (int)rng.size(); b++) glibc_rand_state(seeds[b], rng[b].r, &rng[b].i);
    int32_t bound = initial_bound;
    int32_t overall = initial_bound;
    std::vector<int32_t> seq((size_t)inst->n * inst->m);
    bool have_seq = false;
    std::vector<bsj_beam> beams(num_beams);
    std::vector<bsj_result> res(num_beams);
    std::vector<std::vector<int32_t>> seqs(num_beams, std::vector<int32_t>(seq.size()));
    for (int it = 0; it < iterations; it++) {
        for (int b = 0; b < num_beams; b++) {
            const uint32_t seed = carry ? seeds[b] : seeds[(size_t)it * num_beams + b];
            beams[b] = bsj_beam{mode, beam_width, bound, seed, 0, 0};
            res[b] = bsj_result{};
            res[b].sequence = seqs[b].data();
        }
        bsj_status s = solve_batch_impl(ctx, 1, inst, num_beams, beams.data(), res.data(), stream,
                                        carry ? rng.data() : nullptr, carry ? rng.data() : nullptr);
        if (s != BSJ_OK) return s;
        // MPI_Allreduce(MIN) of the ranks' bests (gpu/v1/main.cu:66-70)
        for (int b = 0; b < num_beams; b++) {
            if (res[b].makespan < overall) {
                overall = res[b].makespan;
                if (res[b].found) { seq = seqs[b]; have_seq = true; }
            }
        }
        bound = overall;
        if (round_best) round_best[it] = overall;
    }
    if (best) *best = overall;
    if (best_sequence) {
        if (have_seq) std::memcpy(best_sequence, seq.data(), seq.size() * sizeof(int32_t));
        else std::memset(best_sequence, 0, seq.size() * sizeof(int32_t));
    }
    return BSJ_OK;
}

}  // extern "C"
