/*
 * bsj.h -- C ABI of the GB300 beam-search engine for the job-shop scheduling problem.
 *
 * Plain C types only (no C++, no torch): pointers, sizes, status codes.  Every call
 * returns a bsj_status; no call exits the process.  Host pointers are borrowed for the
 * duration of the call.  A context owns one device, one stream by default and its device
 * memory; contexts are independent, so several may be used from different threads, but
 * one context (and the plans made from it) is used by one thread at a time.  A server
 * (bsj_server_*) is thread-safe.
 *
 * Reference interfaces these entry points replace (paths within bensdz/BeamSearch_JSSP_GPU):
 *   run_gpu_beam_search_v1   gpu/v1/solver.cuh:6-12, gpu/v1/solver.cu:178-298
 *   run_gpu_beam_search_v2   gpu/v2_twophases/solver.cuh:6-12, gpu/v2_twophases/solver.cu:256-386
 *   beam_search_ich          cpu/v0_ich/solver.h:6, cpu/v0_ich/solver.cpp:8-54
 *   beam_search_pms          cpu/v1_pms/solver.h:6, cpu/v1_pms/solver.cpp:8-70
 *   (the C++ drop-ins with the exact reference signatures are in bsj_solver.h)
 */
#ifndef BSJ_H
#define BSJ_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    BSJ_OK = 0,
    BSJ_ERR_INVALID = 1,   /* malformed argument or instance */
    BSJ_ERR_LIMIT = 2,     /* outside the supported sizes (see BSJ_MAX_*) */
    BSJ_ERR_CUDA = 3,      /* CUDA runtime error; bsj_last_error() has the text */
    BSJ_ERR_NOMEM = 4,     /* device or host allocation failed */
    BSJ_ERR_DEVICE = 5     /* a kernel reported an inconsistent state */
} bsj_status;

/* Search mode of one beam. */
typedef enum {
    BSJ_MODE_V1 = 0,     /* gpu/v1 semantics bit for bit: pivot-machine branching, hash
                            noise, fp32 score, stable order; unscored child slots keep the
                            content of earlier levels (gpu/v1/solver.cu:37-39,73,120,261) */
    BSJ_MODE_V2 = 1,     /* gpu/v2_twophases semantics bit for bit: unscored ranks keep the
                            ping-pong buffer's old state (gpu/v2_twophases/solver.cu:191) */
    BSJ_MODE_CLEAN = 2,  /* same branching, score and order; only scored children compete */
    BSJ_MODE_ICH = 3,    /* cpu/v0_ich: all ready ops, glibc rand() noise, bounded heap */
    BSJ_MODE_PMS = 4     /* cpu/v1_pms: pivot machine from glibc rand(), fp64 score, heap */
} bsj_mode;

#define BSJ_MAX_JOBS 128
#define BSJ_MAX_MACHINES 64
#define BSJ_MAX_OPS 8192
#define BSJ_MAX_BEAM 16384
#define BSJ_MAX_DURATION 16777215
#define BSJ_NO_BOUND 500000   /* the callers' "no bound" value, gpu/v1/main.cu:57 */

/* One instance: n jobs x m machines, job j's k-th op at [j*m + k]; machines 0-based
   (the text format's values, instance_parser.cpp:69-73). Host memory. */
typedef struct {
    int32_t n;
    int32_t m;
    const int32_t *machine;
    const int32_t *duration;
} bsj_instance;

/* One beam (one search pass). */
typedef struct {
    int32_t mode;          /* bsj_mode */
    int32_t beam_width;    /* K, 1..BSJ_MAX_BEAM */
    int32_t best_known;    /* pruning bound; BSJ_NO_BOUND for none */
    uint32_t seed;         /* gpu modes: random_seed; ICH/PMS: the srand() seed */
    int32_t instance;      /* index into the instance array of the batch */
    int32_t bound_group;   /* beams with the same group share one device best-makespan
                              word (atomicMin); -1 = a group of its own */
} bsj_beam;

typedef struct {
    int32_t makespan;      /* the value the reference entry point returns for the mode */
    int32_t found;         /* 1 if a complete schedule was recorded */
    int32_t *sequence;     /* caller-owned [n*m] host buffer or NULL: 1-based op ids
                              (op = job*m + step + 1) in dispatch order */
    int64_t expanded;      /* children scored, summed over levels */
    int64_t slots;         /* child slots considered (P*n for gpu modes) */
    int32_t levels;        /* levels executed */
    int32_t group_best;    /* final value of the beam's bound-group word */
} bsj_result;

typedef struct bsj_context bsj_context;
typedef struct bsj_plan bsj_plan;

/* Version string of the library. */
const char *bsj_version(void);
const char *bsj_status_string(bsj_status s);

/* Number of CUDA devices visible to the process (0 with BSJ_ERR_CUDA when there is no
   usable driver or device). */
bsj_status bsj_device_count(int32_t *count);
/* Context on CUDA device `device` (-1 = current device). */
bsj_status bsj_create(bsj_context **out, int device);
void bsj_destroy(bsj_context *ctx);
/* Text of the last error on this context (valid until the next call). */
const char *bsj_last_error(const bsj_context *ctx);

/* One beam on one instance, synchronous: the C form of run_gpu_beam_search_v1/v2
   (mode V1/V2), beam_search_ich (ICH) and beam_search_pms (PMS).  `stream` is a
   cudaStream_t (NULL = the context's stream). */
bsj_status bsj_solve(bsj_context *ctx, const bsj_instance *inst, const bsj_beam *beam,
                     bsj_result *result, void *stream);

/* Many beams over many instances in one set of launches (independent seeds, batched
   instances of uneven size, mixed modes).  results[i] belongs to beams[i]. */
bsj_status bsj_solve_batch(bsj_context *ctx, int num_instances, const bsj_instance *instances,
                           int num_beams, const bsj_beam *beams, bsj_result *results,
                           void *stream);

/* Multi-start driver with the MPI ranks as beams (gpu/v1/main.cu:58-71,
   cpu/v1_pms/main.cpp:56-67): `iterations` rounds of `num_beams` beams in one launch
   each; a round's beams take, as their pruning bound, the best makespan of all earlier
   rounds and initial_bound (the MPI_Allreduce(MIN), frozen per round).
   Gpu modes: beam b of round i uses random_seed seeds[i*num_beams + b] (what rank b's
   rand() drew for round i).  ICH/PMS: seeds[b] is rank b's srand() seed and its rand()
   stream continues from round to round as the process-wide one does; seeds holds
   num_beams entries.  *best receives the overall best, best_sequence (n*m, may be NULL)
   the schedule of the first beam that reached it (zeros if none beat initial_bound),
   round_best[i] (may be NULL) the best after round i. */
bsj_status bsj_solve_iterations(bsj_context *ctx, const bsj_instance *inst, int mode,
                                int beam_width, int num_beams, int iterations,
                                const uint32_t *seeds, int32_t initial_bound,
                                int32_t *best, int32_t *best_sequence, int32_t *round_best,
                                void *stream);

/* Plans: the split form of bsj_solve_batch used for device-resident timing.
   bsj_plan_create uploads instances and sizes device memory; bsj_plan_run enqueues every
   level on `stream` (asynchronous); bsj_plan_results waits and copies results out. */
bsj_status bsj_plan_create(bsj_context *ctx, int num_instances, const bsj_instance *instances,
                           int num_beams, const bsj_beam *beams, bsj_plan **out);
bsj_status bsj_plan_run(bsj_plan *plan, void *stream);
/* Device bytes bsj_plan_create would allocate for this batch (nothing is allocated);
   errors as bsj_plan_create.  Serving loops admit work against a memory budget with it. */
bsj_status bsj_plan_estimate(bsj_context *ctx, int num_instances, const bsj_instance *instances,
                             int num_beams, const bsj_beam *beams, int64_t *device_bytes);
/* Device bytes a plan holds. */
int64_t bsj_plan_device_bytes(const bsj_plan *plan);
/* New instance data, seeds and bounds into an existing plan, whose captured graph then
   replays without rebuilding: sizes, modes, widths and bound groups must equal the plan's
   (BSJ_ERR_INVALID otherwise).  Not while a run of the plan is in flight. */
bsj_status bsj_plan_update(bsj_plan *plan, int num_instances, const bsj_instance *instances,
                           int num_beams, const bsj_beam *beams);
bsj_status bsj_plan_results(bsj_plan *plan, bsj_result *results);
void bsj_plan_destroy(bsj_plan *plan);
/* Kernel launches one bsj_plan_run enqueues. */
int64_t bsj_plan_launches(const bsj_plan *plan);
/* Algorithmic bytes of the last run, per kernel class: k_step -- per materialised
   survivor one parent snapshot read, one child snapshot written, its 4 B survivor id and
   4 B history entry, plus 8 B per emitted candidate key; k_select -- 8 B per candidate
   key read, 4 B per survivor id written.  Also the run's expanded children, survivors and
   the number of levels whose top-K fell back from the bucket path to the radix path. */
bsj_status bsj_plan_stats(const bsj_plan *plan, double *step_bytes, double *select_bytes,
                          int64_t *expanded, int64_t *materialized, int64_t *select_fallbacks);
/* When enabled, bsj_plan_run records CUDA events around every launch of each kernel
   class; bsj_plan_kernel_ms returns total ms per class and launch counts for the last run:
   index 0 k_step, 1 k_select, 2 k_heap, 3 k_gather_v1, 4 k_finalize. */
bsj_status bsj_plan_set_timing(bsj_plan *plan, int enable);
bsj_status bsj_plan_kernel_ms(const bsj_plan *plan, float *ms, int64_t *launches, int count);

/* ---- Top-K selection routes (no counterpart in the reference, which sorts every slot
   with cub::DeviceRadixSort::SortPairs, gpu/v1/solver.cu:255-258) ----
   The selection kernel of the gpu modes (v1, v2, clean) picks a route per level by its
   size: the direct staged pass, bucket compaction + dense-rank sort, and for rare or
   large levels the radix-select, raw-LSD, rank-LSD, bitonic and large-level routes.  All
   give the same stable (score, slot) order.  bsj_plan_set_select_route forces the plan's
   levels onto routes (BSJ_SELECT_* flags OR'd; 0 = the normal choice), so every route
   can be checked on small inputs; the plan's captured graphs are rebuilt on its next
   run.  Beam groups whose widest gpu-mode beam has K >= 4096 run the selection as a
   cluster of 2 thread blocks per beam (4 where K * n >= 150000), which split the level's
   keys and exchange only summaries through distributed shared memory (route CLUSTER: the
   bucket + dense-rank route on all blocks) on levels of more than 4096 candidate keys;
   smaller levels and those it cannot take fall back to the one-block routes.
   BSJ_SELECT_NO_CLUSTER keeps one block per beam, BSJ_SELECT_FORCE_CLUSTER launches the
   cluster form whatever K and takes its route on every level it can (any size).
   BSJ_SELECT_FORCE_LARGE and BSJ_SELECT_NO_LARGE exclude each other, and so do
   BSJ_SELECT_FORCE_CLUSTER and BSJ_SELECT_NO_CLUSTER; with any other flag set the cluster
   form runs the one-block routes on its first block.
   bsj_plan_select_routes: BSJ_ROUTE_* bits of the routes the last run took (OR over the
   plan's beams and levels; waits for the run). */
#define BSJ_SELECT_FORCE_LARGE 1  /* large-level route (keys read in place) at any size */
#define BSJ_SELECT_NO_LARGE    2  /* never the large-level route */
#define BSJ_SELECT_NO_DIRECT   4  /* compact the survivors first (no direct staged pass) */
#define BSJ_SELECT_RADIX       8  /* MSD radix select of the K-th key (no bucket threshold) */
#define BSJ_SELECT_NO_DENSE    16 /* LSD passes over the raw score bits */
#define BSJ_SELECT_RANK_LSD    32 /* dense ranks written into the keys, then LSD passes */
#define BSJ_SELECT_BITONIC     64 /* block bitonic sort of the survivors */
#define BSJ_SELECT_NO_CLUSTER  128 /* one thread block per beam */
#define BSJ_SELECT_FORCE_CLUSTER 256 /* cluster form and route at any size */
#define BSJ_ROUTE_LARGE    1
#define BSJ_ROUTE_DIRECT   2
#define BSJ_ROUTE_BUCKET   4
#define BSJ_ROUTE_RADIX    8
#define BSJ_ROUTE_DENSE    16
#define BSJ_ROUTE_RANK_LSD 32
#define BSJ_ROUTE_RAW_LSD  64
#define BSJ_ROUTE_BITONIC  128
#define BSJ_ROUTE_CLUSTER  256
bsj_status bsj_plan_set_select_route(bsj_plan *plan, int32_t flags);
bsj_status bsj_plan_select_routes(bsj_plan *plan, uint32_t *routes);
/* enable = 0: one thread block per beam for this plan's selections from its next run on,
   whatever K (a throughput choice: the cluster form spends about twice the SM time per
   level for its lower latency); enable != 0 (the default): the cluster form where the
   rule picks it.  Both forms' graphs are kept, so switching costs one capture per form;
   the results never depend on it.  The route flags above take precedence. */
bsj_status bsj_plan_set_select_cluster(bsj_plan *plan, int32_t enable);

/* ---- Autotuning (no counterpart in the reference, whose launch shape is fixed:
   one block of n threads per parent, gpu/v1/solver.cu:186,237) ----
   The materialise+expand kernel has seven forms ("chunk" codes), and which is fastest
   depends on n, m, K and the number of beams; results never depend on it:
     8, 16, 32   a warp per survivor (the ready list spread over the lanes), 8, 16 or 32
                 consecutive survivors per thread block: small chunks spread a narrow level
                 over more SMs, large ones amortise per-block work;
     1, 2, 3, 4  a group of lanes per survivor (gpu-v2 / clean beams only -- other beams of
                 the group run the warp form of the same chunk): 4 lanes, 32 survivors per
                 block (1, 2) or 8 lanes, 16 per block (3, 4); the parent snapshots staged in
                 shared memory by the group's 16-byte copies (1, 3) or by one bulk copy with
                 an mbarrier (2, 4).  Several times fewer instructions per survivor than the
                 warp form, so beams running side by side contend less.
   Each beam group of a plan (a graph branch) has its own form.  Candidates: 0 = the
   default rule (per group, from the plan's survivors per level, the group's n and
   modes), and each code above for every group.
   bsj_plan_autotune runs the plan once per candidate (an untimed run that also captures
   its graph, then `repeats` timed runs on `stream`, synchronously), keeps the fastest,
   and records it in a process-wide table keyed by device and batch shape, so later plans
   of the same shape (any context, the server included) start with it.  ms (may be NULL)
   receives the mean ms per run of each candidate in the order 0, 8, 16, 32, 1, 2, 3, 4
   (eight floats; a form equal to what the rule gives every group is not run again: its
   entry repeats the rule's); *chunk (may be NULL) the choice.  The plan's results afterwards
   are those of a complete run.  Plans start with the tuned candidate of their shape if
   there is one, else the rule.  bsj_plan_set_chunk selects a candidate; bsj_plan_chunk
   returns it.
   bsj_set_autotune: with enable != 0, bsj_solve_batch / bsj_solve tune every batch shape
   they have not seen on this device before its first solve (about 8 extra solves once
   per shape). */
bsj_status bsj_plan_autotune(bsj_plan *plan, void *stream, int32_t repeats, int32_t *chunk, float *ms);
bsj_status bsj_plan_set_chunk(bsj_plan *plan, int32_t chunk);
int32_t bsj_plan_chunk(const bsj_plan *plan);
bsj_status bsj_set_autotune(bsj_context *ctx, int32_t enable);

/* Instance files in the reference's text format (cpu/common/instance_parser.cpp:8-93).
   bsj_instance_resolve: `arg` as a path, else the reference's Lawrence/Taillard search
   list; BSJ_ERR_INVALID when nothing is found.  bsj_instance_read: *n, *m from the header;
   with machine/duration non-NULL also the [n*m] pairs (machines 0-based, as written),
   BSJ_ERR_LIMIT when n*m > capacity.  A truncated body reads as machine 0 / duration 0,
   as the reference's fscanf loop leaves it. */
bsj_status bsj_instance_resolve(const char *arg, char *out_path, int32_t path_size);
bsj_status bsj_instance_read(const char *path, int32_t *n, int32_t *m, int32_t *machine,
                             int32_t *duration, int32_t capacity);
/* Start times of the semi-active schedule a dispatch order denotes: every op starts at
   max(its machine's ready time, its job predecessor's finish), the rule each search level
   applies (gpu/common/gpu_snapshot.cuh:47-70).  `sequence` holds the n*m 1-based op ids
   of a bsj_result; start[op] (0-based op id, may be NULL) and *makespan receive the
   schedule.  BSJ_ERR_INVALID when the order is not a permutation that keeps every job's
   steps in order. */
bsj_status bsj_schedule_decode(const bsj_instance *inst, const int32_t *sequence, int32_t *start,
                               int32_t *makespan);
/* ---- Serving: continuous batching of independent solves on one GPU ----
   The reference solves one instance per synchronous call.  A server takes requests from
   any number of threads (bsj_submit returns at once), admits queued requests in arrival
   order while an in-flight slot (a CUDA stream) is free and the device memory their plans
   would hold fits the budget, runs each as one CUDA-graph launch so that requests overlap
   on the device, and reuses finished plans for later requests of the same shape.  Each
   request is one beam (bound_group is ignored); its result equals bsj_solve's. */
typedef struct bsj_server bsj_server;
typedef struct {
    int32_t max_inflight;    /* requests on the device at once; 0 = 32, at most 256 */
    int32_t cluster_inflight; /* a request runs the cluster select (K >= 4096) only when at
                                most this many others are in flight at its admission:
                                0 = the device's SMs / 8, < 0 = never */
    int64_t memory_budget;   /* device bytes held by running and idle plans; 0 = 3/4 of
                                the free memory at creation */
} bsj_server_config;
typedef struct {
    double queue_ms;         /* submit -> admission */
    double run_ms;           /* admission -> completion seen by the server */
    int32_t built_plan;      /* 1 if no idle plan of the request's shape was free and the
                                server built one (allocation + graph capture on its run) */
    int32_t reserved;
} bsj_request_times;
typedef struct {
    int64_t submitted, completed;
    int64_t plans_built, plans_reused;
    int64_t peak_inflight;
    int64_t peak_device_bytes;
    int64_t budget_bytes;
    int64_t pending;
    /* host time the server's worker spent, summed over requests (ms): building new plans
       (allocation + graph capture on first run), loading requests into reused plans,
       launching, and collecting results */
    double build_ms, update_ms, launch_ms, collect_ms;
    int64_t plans_prepared;  /* plans built by bsj_server_prepare and now in the idle pool
                                (included in plans_built) */
} bsj_server_stats;
/* cfg may be NULL (defaults). */
bsj_status bsj_server_create(bsj_server **out, int device, const bsj_server_config *cfg);
/* Drops queued requests, waits for running ones, frees everything.  No other thread may
   be inside a call on this server (a bsj_wait on a dropped request would never return). */
void bsj_server_destroy(bsj_server *server);
/* Copies the request and queues it.  BSJ_ERR_INVALID / BSJ_ERR_LIMIT as bsj_solve would
   return them, and BSJ_ERR_LIMIT when the request alone exceeds the memory budget. */
bsj_status bsj_submit(bsj_server *server, const bsj_instance *inst, const bsj_beam *beam,
                      uint64_t *ticket);
/* Non-blocking: *done = 0 while the request is queued or running; once *done = 1 the
   result (the sequence copied into result->sequence when non-NULL), its times and its
   status are handed out and the ticket is retired.  BSJ_ERR_INVALID for unknown tickets. */
bsj_status bsj_poll(bsj_server *server, uint64_t ticket, bsj_result *result,
                    bsj_request_times *times, int32_t *done);
/* Blocking form of bsj_poll. */
bsj_status bsj_wait(bsj_server *server, uint64_t ticket, bsj_result *result,
                    bsj_request_times *times);
bsj_status bsj_server_get_stats(bsj_server *server, bsj_server_stats *out);
/* Builds `copies` plans of the shape of (inst, beam) -- n, m, mode, K -- ahead of the
   requests that will need them: each is created, run once on `inst` (which captures its
   graph) and kept in the idle pool, so requests of that shape arriving later reuse a
   ready plan instead of building one while they wait.  Queued behind earlier requests
   and handled by the worker like them, within the memory budget (idle plans remain
   subject to eviction when memory is short); produces no result.  Errors as bsj_submit.
   A long-running server calls it once per shape it expects, before traffic arrives. */
bsj_status bsj_server_prepare(bsj_server *server, const bsj_instance *inst, const bsj_beam *beam,
                              int32_t copies);

/* Single-beam solve that allocates nothing (no counterpart in the reference).
   For callers that must not allocate device memory -- operator/plugin hosts whose device
   memory is owned and budgeted by the host framework, and latency-critical loops where a
   cudaMalloc/cudaFree would synchronise the device or could fail mid-run.  It needs no
   context: all intermediate state lives in one library-owned scratch array of
   BSJ_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until exit.
     d_machine, d_duration  device [n*m] int32 (machines 0-based), read only
     mode                   BSJ_MODE_V2 or BSJ_MODE_CLEAN
     d_out                  device [2 + n*m] int32: makespan, found, then the 1-based op
                            sequence.  The makespan is -1 (found 0, sequence zeros) if
                            the instance holds a machine id outside [0,m), a duration
                            outside [0,2^24), or durations summing to 2^31-1 or more;
                            it is -2 (found 0, sequence zeros) if a device consistency
                            check of the level kernels failed (what bsj_solve reports
                            as BSJ_ERR_DEVICE)
   Asynchronous on `stream` (a cudaStream_t, NULL = default stream): the call only
   enqueues kernels and a memset and reads no host memory on the stream.  Returns
   BSJ_ERR_LIMIT when n, m, beam_width exceed the BSJ_MAX_* limits or the beam's working
   set (about 2*K*(4m+6n+16) + 10*K*n + 4*K*n*m bytes) exceeds the scratch array.  The
   first call on each device looks up the scratch array's device address: make it before
   any stream capture.  Calls share the scratch array: calls that overlap on one GPU race
   and must be serialised by the caller. */
#define BSJ_NOALLOC_SCRATCH_BYTES (64u << 20)
bsj_status bsj_solve_noalloc(int32_t n, int32_t m, const int32_t *d_machine,
                             const int32_t *d_duration, int32_t mode, int32_t beam_width,
                             int32_t best_known, uint32_t seed, int32_t *d_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
