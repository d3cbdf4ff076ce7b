/*
 * bsj_oracle.c -- CPU oracle for the JSSP beam-search level.
 *
 * TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py as the checker / CPU reference.  The product library
 * (beamsearch_jssp_gpu_gb300/csrc) never links or calls it.
 *
 * The state is kept in the reference's own representation (1-based machine ids, op ids
 * 1..N with dummies 0 and N+1, a finish time per op, an ordered ready list and the op
 * sequence) so that this restatement is independent of the compact layout the CUDA path
 * uses.  Every function cites the reference file:line it follows.
 *
 * Pinning: ORC_ICH and ORC_PMS are checked bit-for-bit (makespan) against the reference
 * CPU solvers compiled from their own sources (oracle/Makefile -> oracle/_ref); the gpu
 * modes are checked against the reference gpu kernels run on the GPU (fixtures under
 * tests/golden/).
 */
#include "bsj_oracle.h"

#include <stdlib.h>
#include <string.h>

#define SENTINEL 500000          /* "no bound" value used by every reference caller */
#define MARK 0xFFFFFFFFu         /* trace value for a rank that was not rewritten */
#define FILLER_SCORE 1e9f        /* gpu/v1/solver.cu:37, gpu/v2_twophases/solver.cu:34 */

/* ------------------------------------------------------------------------------------ */
/* glibc rand(): additive feedback generator r[i] = r[i-31] + r[i-3] (mod 2^32), seeded  */
/* by the Park-Miller LCG (16807, 2^31-1) through Schrage's method, 310 outputs          */
/* discarded, output r[i] >> 1.  (Published algorithm of glibc random_r.c TYPE_3, the    */
/* generator behind srand(12345) in cpu/v0_ich/main.cpp:39 and the rand() draws of       */
/* cpu/v0_ich/solver.cpp:35, cpu/v1_pms/solver.cpp:32,52.)                               */
/* ------------------------------------------------------------------------------------ */
typedef struct {
    uint32_t r[34];
    unsigned i;  /* index of the next value in the conceptual sequence r[] */
} grand_t;

static void grand_seed(grand_t *g, uint32_t seed)
{
    uint32_t r[344];
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
    for (int k = 310; k < 344; k++) g->r[k % 34] = r[k];
    g->i = 344;
}

static int32_t grand_next(grand_t *g)
{
    unsigned i = g->i;
    uint32_t v = g->r[(i - 31) % 34] + g->r[(i - 3) % 34];
    g->r[i % 34] = v;
    g->i = i + 1;
    return (int32_t)(v >> 1);
}

void orc_glibc_rand_fill(uint32_t seed, int32_t *out, int count)
{
    grand_t g;
    grand_seed(&g, seed);
    for (int k = 0; k < count; k++) out[k] = grand_next(&g);
}

/* ------------------------------------------------------------------------------------ */
/* gpu-mode hashes and score (gpu/v1/solver.cu:51-54, :121-126; v2 :47-50, :117-122)     */
/* ------------------------------------------------------------------------------------ */
uint32_t orc_pivot_hash(uint32_t h)
{
    h ^= h >> 16; h *= 0x7feb352du;
    h ^= h >> 15; h *= 0x846ca68bu;
    h ^= h >> 16;
    return h;
}

uint32_t orc_noise_hash(uint32_t seed, uint32_t c, uint32_t b)
{
    uint32_t h = seed ^ (c * 0x85ebca6bu) ^ (b * 0xc2b2ae35u);
    h ^= h >> 16; h *= 0x85ebca6bu;
    h ^= h >> 16; h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

float orc_gpu_score(int32_t cmax, int32_t num_scheduled, uint32_t seed, uint32_t c, uint32_t b)
{
    volatile float base = (num_scheduled == 0) ? (float)cmax : ((float)cmax / (float)num_scheduled);
    volatile float noise = (float)(orc_noise_hash(seed, c, b) % 1000u) / 1000000000.0f;
    return base + noise;
}

/* ------------------------------------------------------------------------------------ */
/* State in the reference's representation (cpu/common/jssp_types.h:26-37,               */
/* gpu/common/gpu_snapshot.cuh:8-31).                                                    */
/* ------------------------------------------------------------------------------------ */
typedef struct {
    int32_t *tr;      /* [m+1] machine ready time, 1-based machines */
    int32_t *tf;      /* [N+2] finish time per op id */
    int32_t *ready;   /* [n]   ready op ids, order significant */
    int32_t *seq;     /* [N]   scheduled op ids */
    int32_t nready, nseq, cmax;
    double score;
    uint32_t lineage; /* (parent rank << 8) | job of the child that produced this state */
    int32_t stamp;    /* step+1 at which this state was written, 0 = never */
} ost;

typedef struct {
    int n, m, N, ints;
    const int32_t *mc, *du;
} octx;

static int32_t op_machine1(const octx *x, int op) { return x->mc[op - 1] + 1; }
static int32_t op_dur(const octx *x, int op) { return x->du[op - 1]; }
static int32_t op_job(const octx *x, int op) { return (op - 1) / x->m; }

typedef struct {
    ost *st;
    int32_t *mem;
    int count;
} opool;

static int pool_init(opool *p, const octx *x, int count)
{
    p->count = count;
    p->st = (ost *)calloc((size_t)count, sizeof(ost));
    p->mem = (int32_t *)calloc((size_t)count * (size_t)x->ints, sizeof(int32_t));
    if (!p->st || !p->mem) return -1;
    for (int k = 0; k < count; k++) {
        int32_t *b = p->mem + (size_t)k * x->ints;
        p->st[k].tr = b;
        p->st[k].tf = b + (x->m + 1);
        p->st[k].ready = p->st[k].tf + (x->N + 2);
        p->st[k].seq = p->st[k].ready + x->n;
    }
    return 0;
}

static void pool_free(opool *p)
{
    free(p->st);
    free(p->mem);
    p->st = NULL;
    p->mem = NULL;
}

static void st_copy(const octx *x, ost *d, const ost *s)
{
    memcpy(d->tr, s->tr, (size_t)x->ints * sizeof(int32_t));
    d->nready = s->nready;
    d->nseq = s->nseq;
    d->cmax = s->cmax;
    d->score = s->score;
    d->lineage = s->lineage;
    d->stamp = s->stamp;
}

/* Root: first op of every job ready in job order (jssp_types.h:61-72,
   gpu_snapshot.cuh:34-44). */
static void st_root(const octx *x, ost *s)
{
    memset(s->tr, 0, (size_t)x->ints * sizeof(int32_t));
    for (int j = 0; j < x->n; j++) s->ready[j] = j * x->m + 1;
    s->nready = x->n;
    s->nseq = 0;
    s->cmax = 0;
    s->score = 0.0;
    s->lineage = MARK;
    s->stamp = 0;
}

/* schedule_operation (jssp_types.h:75-97) == dev_schedule_operation
   (gpu_snapshot.cuh:47-70) followed by the makespan loop (gpu/v1/solver.cu:114-117).
   The caller has already removed `op` from the ready list. */
static void st_schedule(const octx *x, ost *s, int op)
{
    const int M = x->m;
    int mc = op_machine1(x, op);
    s->seq[s->nseq++] = op;
    int pred = (op % M == 1) ? 0 : s->tf[op - 1];
    int start = s->tr[mc] > pred ? s->tr[mc] : pred;
    s->tr[mc] = start + op_dur(x, op);
    s->tf[op] = s->tr[mc];
    if (op % M != 0) s->ready[s->nready++] = op + 1;
    int cmax = 0;
    for (int k = 1; k <= M; k++)
        if (s->tr[k] > cmax) cmax = s->tr[k];
    s->cmax = cmax;
}

/* Swap-with-last removal (gpu/v1/solver.cu:100-106, v2 :96-102). */
static void st_remove_swap(ost *s, int op)
{
    for (int i = 0; i < s->nready; i++) {
        if (s->ready[i] == op) {
            s->ready[i] = s->ready[--s->nready];
            break;
        }
    }
}

/* Order-preserving erase at position idx (cpu/v0_ich/solver.cpp:29,
   cpu/v1_pms/solver.cpp:44-46). */
static void st_erase_at(ost *s, int idx)
{
    for (int i = idx; i + 1 < s->nready; i++) s->ready[i] = s->ready[i + 1];
    s->nready--;
}

/* ------------------------------------------------------------------------------------ */
/* Bounded max-heap beam (cpu/common/jssp_types.h:40-58) with the hole-based sift steps  */
/* of libstdc++'s std::push_heap / std::pop_heap, whose layout decides both which state  */
/* is evicted among equal scores and the next level's parent order.                    */
/* ------------------------------------------------------------------------------------ */
static int heap_less(const ost *a, const ost *b) { return a->score < b->score; }

static void heap_sift_up(ost **a, int hole, int top, ost *value)
{
    int parent = (hole - 1) / 2;
    while (hole > top && heap_less(a[parent], value)) {
        a[hole] = a[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    a[hole] = value;
}

static void heap_push(ost **a, int len) { heap_sift_up(a, len - 1, 0, a[len - 1]); }

static void heap_adjust(ost **a, int hole, int len, ost *value)
{
    const int top = hole;
    int child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (heap_less(a[child], a[child - 1])) child--;
        a[hole] = a[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        a[hole] = a[child - 1];
        hole = child - 1;
    }
    heap_sift_up(a, hole, top, value);
}

static void heap_pop(ost **a, int len)
{
    if (len > 1) {
        ost *value = a[len - 1];
        a[len - 1] = a[0];
        heap_adjust(a, 0, len - 1, value);
    }
}

typedef struct {
    ost **arr;   /* heap array, size <= K */
    int size, K;
    ost *spare;  /* buffer the next child is built in */
    ost **free_list;
    int nfree;
} obeam;

/* insert_into_beam (jssp_types.h:47-58): `child` lives in b->spare. */
static void beam_insert(obeam *b)
{
    ost *child = b->spare;
    if (b->size < b->K) {
        b->arr[b->size++] = child;
        heap_push(b->arr, b->size);
        b->spare = b->nfree > 0 ? b->free_list[--b->nfree] : NULL;
    } else if (child->score < b->arr[0]->score) {
        heap_pop(b->arr, b->size);
        ost *evicted = b->arr[b->size - 1];
        b->arr[b->size - 1] = child;
        heap_push(b->arr, b->size);
        b->spare = evicted;
    }
}

/* ------------------------------------------------------------------------------------ */
/* gpu v1 / v2 / clean level loop (gpu/v1/solver.cu:178-298, :9-176;                    */
/* gpu/v2_twophases/solver.cu:256-386, :9-254).                                          */
/* ------------------------------------------------------------------------------------ */
typedef struct { float key; int32_t idx; } skey;

static int skey_cmp(const void *pa, const void *pb)
{
    const skey *a = (const skey *)pa, *b = (const skey *)pb;
    if (a->key < b->key) return -1;
    if (a->key > b->key) return 1;
    return (a->idx > b->idx) - (a->idx < b->idx);  /* stable: slot order among ties */
}

static int solve_gpu(const octx *x, const orc_params *p, orc_result *res, int max_levels)
{
    const int n = x->n, N = x->N, K = p->beam_width, mode = p->mode;
    const size_t maxc = (size_t)K * (size_t)n;
    opool pa = {0}, pb = {0}, ps = {0}, pt = {0};
    int rc = -1;
    skey *keys = (skey *)malloc(maxc * sizeof(skey));
    int32_t *cand = (int32_t *)malloc(maxc * sizeof(int32_t));
    int32_t *cnt = (int32_t *)malloc((size_t)K * sizeof(int32_t));
    int32_t *best_seq = (int32_t *)calloc((size_t)N, sizeof(int32_t));
    if (!keys || !cand || !cnt || !best_seq) goto out;
    if (pool_init(&pa, x, K) || pool_init(&pb, x, K) || pool_init(&pt, x, 1)) goto out;
    if (mode == ORC_GPU_V1 && pool_init(&ps, x, (int)maxc)) goto out;

    ost *cur = pa.st, *nxt = pb.st, *tmp = pt.st;
    st_root(x, &cur[0]);
    int P = 1;
    const int bound = p->best_known;
    uint64_t best_key = UINT64_MAX;
    int levels = 0, ties = 0;
    res->expanded = 0;
    res->slots = 0;

    for (int s = 0; s < N && s < max_levels; s++) {
        const uint32_t seed_s = p->seed + (uint32_t)s;
        const int total = P * n;
        int scored = 0;
        levels++;
        res->slots += total;
        for (int c = 0; c < P; c++) {
            const ost *par = &cur[c];
            int count = 0;
            /* pivot machine (gpu/v1/solver.cu:47-69) */
            if (par->nready > 0) {
                uint32_t h = orc_pivot_hash(seed_s + (uint32_t)c);
                int chosen = par->ready[h % (uint32_t)par->nready];
                int cm = op_machine1(x, chosen);
                for (int i = 0; i < par->nready; i++)
                    if (op_machine1(x, par->ready[i]) == cm) cand[(size_t)c * n + count++] = par->ready[i];
            }
            cnt[c] = count;
            for (int b = 0; b < n; b++) {
                keys[(size_t)c * n + b].key = FILLER_SCORE;
                keys[(size_t)c * n + b].idx = c * n + b;
            }
            for (int b = 0; b < count; b++) {
                int op = cand[(size_t)c * n + b];
                st_copy(x, tmp, par);
                st_remove_swap(tmp, op);
                st_schedule(x, tmp, op);
                /* prune against the bound (gpu/v1/solver.cu:120); before the last step the
                   device bound still equals best_known */
                if (tmp->cmax < bound) {
                    keys[(size_t)c * n + b].key =
                        orc_gpu_score(tmp->cmax, tmp->nseq, seed_s, (uint32_t)c, (uint32_t)b);
                    scored++;
                    if (mode == ORC_GPU_V1) {
                        ost *slot = &ps.st[(size_t)c * n + b];
                        st_copy(x, slot, tmp);
                        slot->lineage = ((uint32_t)c << 8) | (uint32_t)op_job(x, op);
                        slot->stamp = s + 1;
                    }
                    /* complete solution (gpu/v1/solver.cu:147-155): deterministic choice of
                       min (cmax, slot) for the reference's racy copy */
                    if (tmp->nseq == N) {
                        uint64_t kk = ((uint64_t)(uint32_t)tmp->cmax << 32) | (uint32_t)(c * n + b);
                        if (best_key == UINT64_MAX || tmp->cmax < (int)(best_key >> 32)) ties = 0;
                        if (kk < best_key) {
                            best_key = kk;
                            memcpy(best_seq, tmp->seq, (size_t)N * sizeof(int32_t));
                        }
                        if (tmp->cmax == (int)(best_key >> 32)) {
                            if (p->ties && ties < p->max_ties)
                                memcpy(p->ties + (size_t)ties * N, tmp->seq, (size_t)N * sizeof(int32_t));
                            ties++;
                        }
                    }
                }
            }
        }
        res->expanded += scored;
        if (s == N - 1) break;  /* the last sort/gather is not observable */

        /* stable ascending sort of all P*n slots (gpu/v1/solver.cu:255-258) */
        qsort(keys, (size_t)total, sizeof(skey), skey_cmp);
        int keff = total < K ? total : K;
        if (mode == ORC_GPU_CLEAN) keff = scored < K ? scored : K;

        if (mode == ORC_GPU_V1) {
            /* kernel_gather_topk (gpu/v1/solver.cu:160-176): copy whatever the slot holds */
            for (int r = 0; r < keff; r++) {
                const ost *slot = &ps.st[keys[r].idx];
                st_copy(x, &cur[r], slot);
                if (p->trace)
                    p->trace[(size_t)s * K + r] = (slot->stamp == s + 1) ? slot->lineage : MARK;
            }
        } else {
            /* kernel_materialize_topk (gpu/v2_twophases/solver.cu:150-254): ranks whose
               branch is not a candidate keep the ping-pong buffer's old content (:191) */
            for (int r = 0; r < keff; r++) {
                int c = keys[r].idx / n, b = keys[r].idx % n;
                if (b >= cnt[c]) {
                    if (p->trace) p->trace[(size_t)s * K + r] = MARK;
                    continue;
                }
                int op = cand[(size_t)c * n + b];
                st_copy(x, &nxt[r], &cur[c]);
                st_remove_swap(&nxt[r], op);
                st_schedule(x, &nxt[r], op);
                nxt[r].lineage = ((uint32_t)c << 8) | (uint32_t)op_job(x, op);
                nxt[r].stamp = s + 1;
                if (p->trace) p->trace[(size_t)s * K + r] = nxt[r].lineage;
            }
            ost *sw = cur; cur = nxt; nxt = sw;
        }
        if (p->trace_count) p->trace_count[s] = keff;
        P = keff;
        if (P == 0) break;
    }

    res->levels = levels;
    res->ties = ties;
    if (best_key != UINT64_MAX) {
        int cm = (int)(best_key >> 32);
        res->makespan = cm < bound ? cm : bound;
        res->found = 1;
        if (res->seq) memcpy(res->seq, best_seq, (size_t)N * sizeof(int32_t));
    } else {
        res->makespan = bound;
        res->found = 0;
        /* the reference copies its never-written best buffer when bound < 500000
           (gpu/v1/solver.cu:280-284); a fresh allocation reads as zeros */
        if (res->seq) memset(res->seq, 0, (size_t)N * sizeof(int32_t));
    }
    rc = 0;
out:
    pool_free(&pa); pool_free(&pb); pool_free(&ps); pool_free(&pt);
    free(keys); free(cand); free(cnt); free(best_seq);
    return rc;
}

/* ------------------------------------------------------------------------------------ */
/* BS-ICH (cpu/v0_ich/solver.cpp:8-54) and BS-PMS (cpu/v1_pms/solver.cpp:8-70)          */
/* ------------------------------------------------------------------------------------ */
static int beam_init(obeam *b, opool *pool, int K)
{
    b->K = K;
    b->size = 0;
    b->arr = (ost **)malloc((size_t)(K + 1) * sizeof(ost *));
    b->free_list = (ost **)malloc((size_t)(K + 1) * sizeof(ost *));
    if (!b->arr || !b->free_list) return -1;
    b->nfree = 0;
    for (int k = pool->count - 1; k >= 1; k--) b->free_list[b->nfree++] = &pool->st[k];
    b->spare = &pool->st[0];
    return 0;
}

static void beam_reset(obeam *b, opool *pool)
{
    b->size = 0;
    b->nfree = 0;
    for (int k = pool->count - 1; k >= 1; k--) b->free_list[b->nfree++] = &pool->st[k];
    b->spare = &pool->st[0];
}

/* `carry` (may be NULL): the rand() stream to draw from, left where the pass ends, as the
   process-wide state is between the reference's successive calls (cpu/v1_pms/main.cpp:56,64);
   NULL seeds a fresh stream with p->seed. */
static int solve_cpu(const octx *x, const orc_params *p, orc_result *res, int max_levels,
                     grand_t *carry)
{
    const int N = x->N, K = p->beam_width, mode = p->mode;
    opool pool[2] = {{0}, {0}};
    obeam beam[2] = {{0}, {0}};
    int rc = -1;
    int32_t *best_seq = (int32_t *)calloc((size_t)N, sizeof(int32_t));
    if (!best_seq) goto out;
    if (pool_init(&pool[0], x, K + 1) || pool_init(&pool[1], x, K + 1)) goto out;
    if (beam_init(&beam[0], &pool[0], K) || beam_init(&beam[1], &pool[1], K)) goto out;

    grand_t own;
    if (!carry) grand_seed(&own, p->seed);
    grand_t *gp = carry ? carry : &own;
    int cb = 0;
    /* the initial beam holds the root */
    st_root(x, beam[cb].spare);
    beam[cb].arr[0] = beam[cb].spare;
    beam[cb].size = 1;
    beam[cb].spare = beam[cb].free_list[--beam[cb].nfree];

    int best_mk = SENTINEL;
    int levels = 0;
    res->expanded = 0;
    res->slots = 0;
    const int max_steps = (mode == ORC_ICH) ? N : N + 10;  /* v0_ich :19; v1_pms :23 */
    for (int s = 0; s < max_steps && s < max_levels && beam[cb].size > 0; s++) {
        obeam *cur = &beam[cb], *nb = &beam[cb ^ 1];
        beam_reset(nb, &pool[cb ^ 1]);
        if (s < N) levels++;
        for (int c = 0; c < cur->size; c++) {
            const ost *par = cur->arr[c];
            if (mode == ORC_ICH) {
                for (int idx = 0; idx < par->nready; idx++) {
                    ost *child = nb->spare;
                    int op = par->ready[idx];
                    st_copy(x, child, par);
                    st_erase_at(child, idx);
                    st_schedule(x, child, op);
                    child->score = (double)child->cmax + (grand_next(gp) % 100) * 0.01;
                    child->lineage = ((uint32_t)c << 8) | (uint32_t)op_job(x, op);
                    res->expanded++;
                    res->slots++;
                    beam_insert(nb);
                }
            } else {
                int nbr = par->nready;
                if (nbr <= 0) continue;
                int pivot = grand_next(gp) % nbr;
                int target = op_machine1(x, par->ready[pivot]);
                for (int r = 0; r < nbr; r++) {
                    if (op_machine1(x, par->ready[r]) != target) continue;
                    ost *child = nb->spare;
                    int op = par->ready[r];
                    st_copy(x, child, par);
                    for (int i = 0; i < child->nready; i++) {
                        if (child->ready[i] == op) { st_erase_at(child, i); break; }
                    }
                    st_schedule(x, child, op);
                    double noise = (double)(grand_next(gp) % 1000) / 1000000.0;
                    child->score = ((double)child->cmax / (double)child->nseq) + noise;
                    child->lineage = ((uint32_t)c << 8) | (uint32_t)op_job(x, op);
                    res->expanded++;
                    res->slots++;
                    if (child->nseq == N && child->cmax < best_mk) {
                        best_mk = child->cmax;
                        memcpy(best_seq, child->seq, (size_t)N * sizeof(int32_t));
                    }
                    if (child->cmax < p->best_known) beam_insert(nb);
                }
            }
        }
        if (p->trace && s < N) {
            for (int r = 0; r < nb->size; r++) p->trace[(size_t)s * K + r] = nb->arr[r]->lineage;
        }
        if (p->trace_count && s < N) p->trace_count[s] = nb->size;
        cb ^= 1;
    }
    res->levels = levels;
    res->ties = 0;
    if (mode == ORC_ICH) {
        /* min cmax over the final beam, first in array order (v0_ich/solver.cpp:47-51) */
        int best = SENTINEL;
        const obeam *fb = &beam[cb];
        const ost *bs = NULL;
        for (int r = 0; r < fb->size; r++)
            if (fb->arr[r]->cmax < best) { best = fb->arr[r]->cmax; bs = fb->arr[r]; }
        res->makespan = best;
        res->found = (bs != NULL && bs->nseq == N);
        if (res->seq) {
            if (bs) memcpy(res->seq, bs->seq, (size_t)N * sizeof(int32_t));
            else memset(res->seq, 0, (size_t)N * sizeof(int32_t));
        }
    } else {
        res->makespan = best_mk;
        res->found = best_mk < SENTINEL;
        if (res->seq) memcpy(res->seq, best_seq, (size_t)N * sizeof(int32_t));
    }
    rc = 0;
out:
    for (int k = 0; k < 2; k++) {
        free(beam[k].arr);
        free(beam[k].free_list);
        pool_free(&pool[k]);
    }
    free(best_seq);
    return rc;
}

static int solve_any(const orc_instance *inst, const orc_params *p, orc_result *res,
                     int max_levels, grand_t *carry)
{
    if (!inst || !p || !res) return -1;
    if (inst->n < 1 || inst->m < 1 || inst->n > 255 || p->beam_width < 1) return -2;
    for (int k = 0; k < inst->n * inst->m; k++)
        if (inst->machine[k] < 0 || inst->machine[k] >= inst->m || inst->duration[k] < 0) return -3;
    octx x;
    x.n = inst->n;
    x.m = inst->m;
    x.N = inst->n * inst->m;
    x.ints = (x.m + 1) + (x.N + 2) + x.n + x.N;
    x.mc = inst->machine;
    x.du = inst->duration;
    switch (p->mode) {
    case ORC_GPU_V1:
    case ORC_GPU_V2:
    case ORC_GPU_CLEAN:
        return solve_gpu(&x, p, res, max_levels);
    case ORC_ICH:
    case ORC_PMS:
        return solve_cpu(&x, p, res, max_levels, carry);
    default:
        return -4;
    }
}

int orc_solve_levels(const orc_instance *inst, const orc_params *p, orc_result *res,
                     int max_levels)
{
    return solve_any(inst, p, res, max_levels, NULL);
}

/* Multi-start loop of the reference drivers with the MPI ranks as beams: gpu/v1/main.cu:58-71
   (each rank draws a random_seed per round, calls the solver with the all-reduced bound,
   then MPI_Allreduce(MIN)) and cpu/v1_pms/main.cpp:56-67 (srand once per rank, the rand()
   stream runs on across rounds). */
int orc_solve_iterations(const orc_instance *inst, int mode, int K, int num_beams, int iterations,
                         const uint32_t *seeds, int32_t initial_bound, int32_t *best,
                         int32_t *best_seq, int32_t *round_best)
{
    if (!inst || !seeds || num_beams < 1 || iterations < 1) return -1;
    const int N = inst->n * inst->m;
    const int cpu = (mode == ORC_ICH || mode == ORC_PMS);
    grand_t *streams = (grand_t *)malloc((size_t)num_beams * sizeof(grand_t));
    int32_t *seq = (int32_t *)malloc((size_t)N * sizeof(int32_t));
    if (!streams || !seq) { free(streams); free(seq); return -1; }
    if (cpu)
        for (int b = 0; b < num_beams; b++) grand_seed(&streams[b], seeds[b]);
    int32_t overall = initial_bound, bound = initial_bound;
    int have = 0, rc = 0;
    for (int it = 0; it < iterations && rc == 0; it++) {
        for (int b = 0; b < num_beams; b++) {
            orc_params p;
            memset(&p, 0, sizeof(p));
            p.mode = mode;
            p.beam_width = K;
            p.best_known = bound;
            p.seed = cpu ? seeds[b] : seeds[(size_t)it * num_beams + b];
            orc_result r;
            memset(&r, 0, sizeof(r));
            r.seq = seq;
            rc = solve_any(inst, &p, &r, 1 << 30, cpu ? &streams[b] : NULL);
            if (rc != 0) break;
            if (r.makespan < overall) {
                overall = r.makespan;
                if (r.found && best_seq) { memcpy(best_seq, seq, (size_t)N * sizeof(int32_t)); have = 1; }
            }
        }
        bound = overall;
        if (round_best) round_best[it] = overall;
    }
    if (rc == 0) {
        if (best) *best = overall;
        if (best_seq && !have) memset(best_seq, 0, (size_t)N * sizeof(int32_t));
    }
    free(streams);
    free(seq);
    return rc;
}

int orc_solve(const orc_instance *inst, const orc_params *p, orc_result *res)
{
    return orc_solve_levels(inst, p, res, 1 << 30);
}

int32_t orc_schedule_makespan(const orc_instance *inst, const int32_t *seq)
{
    const int n = inst->n, m = inst->m, N = n * m;
    int32_t *tr = (int32_t *)calloc((size_t)m, sizeof(int32_t));
    int32_t *jr = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    int32_t *nx = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    int32_t cmax = 0;
    if (!tr || !jr || !nx) { cmax = -1; goto out; }
    for (int t = 0; t < N; t++) {
        int op = seq[t];
        if (op < 1 || op > N) { cmax = -1; goto out; }
        int j = (op - 1) / m, k = (op - 1) % m;
        if (k != nx[j]) { cmax = -1; goto out; }
        int mc = inst->machine[j * m + k];
        int start = tr[mc] > jr[j] ? tr[mc] : jr[j];
        int fin = start + inst->duration[j * m + k];
        tr[mc] = fin;
        jr[j] = fin;
        nx[j]++;
        if (fin > cmax) cmax = fin;
    }
out:
    free(tr); free(jr); free(nx);
    return cmax;
}
