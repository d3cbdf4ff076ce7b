/*
 * bsj_oracle.h -- CPU oracle for the JSSP beam-search level (TEST INFRASTRUCTURE ONLY).
 *
 * This header and bsj_oracle.c restate, in plain C, the algorithms of the reference
 * solvers so that tests, smoke() and the CPU-baseline leg of bench.py can check and time
 * the CUDA path.  Nothing in the product library links or calls this code.
 *
 * Modes (all follow the reference file:line cited in bsj_oracle.c):
 *   ORC_GPU_V1    gpu/v1/solver.cu semantics, including the stale child-slot reuse
 *   ORC_GPU_V2    gpu/v2_twophases/solver.cu semantics, including stale ping-pong ranks
 *   ORC_GPU_CLEAN same branching/score/order as the gpu solvers, only valid children compete
 *   ORC_ICH       cpu/v0_ich/solver.cpp (glibc rand() noise, libstdc++ bounded heap)
 *   ORC_PMS       cpu/v1_pms/solver.cpp (glibc rand() pivot + noise, bounded heap)
 */
#ifndef BSJ_ORACLE_H
#define BSJ_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_GPU_V1 = 0, ORC_GPU_V2 = 1, ORC_GPU_CLEAN = 2, ORC_ICH = 3, ORC_PMS = 4 };

/* Instance: n jobs x m machines; op (job j, step k) at index j*m+k, machines 0-based. */
typedef struct {
    int n, m;
    const int32_t *machine;
    const int32_t *duration;
} orc_instance;

typedef struct {
    int mode;
    int beam_width;      /* K */
    int best_known;      /* pruning bound (500000 = none) */
    uint32_t seed;       /* gpu modes: random_seed; ICH/PMS: srand() seed */
    /* optional per-level trace: trace[s*K + r] = (parent_rank << 8) | job of the state
       placed at rank r of the beam after step s, 0xFFFFFFFF where the rank was not
       rewritten at that step; trace_count[s] = beam size after step s. */
    uint32_t *trace;
    int32_t *trace_count;
    /* optional (gpu modes): schedules of the complete children that tie for the best
       makespan, up to max_ties of them, [max_ties][n*m]; count in orc_result.ties */
    int32_t *ties;
    int32_t max_ties;
} orc_params;

typedef struct {
    int32_t makespan;     /* the value the reference entry point returns */
    int32_t found;        /* 1 if a complete schedule was recorded */
    int32_t *seq;         /* caller-owned [n*m]: 1-based op ids of the best schedule */
    int64_t expanded;     /* children scored (valid, unpruned) summed over levels */
    int64_t slots;        /* P*n (gpu modes) or children generated (ICH/PMS) summed */
    int32_t levels;       /* levels that expanded at least one parent */
    int32_t ties;         /* complete children with the best makespan (gpu modes) */
} orc_result;

/* Returns 0 on success, negative on invalid input / allocation failure. */
int orc_solve(const orc_instance *inst, const orc_params *p, orc_result *res);

/* Solve only the first `max_levels` levels (CPU baseline sample); result fields are
   filled for the levels executed. */
int orc_solve_levels(const orc_instance *inst, const orc_params *p, orc_result *res,
                     int max_levels);

/* Multi-start loop with the ranks as beams (gpu/v1/main.cu:58-71, cpu/v1_pms/main.cpp:56-67):
   round it's beams get the best of all earlier rounds as bound.  gpu modes: beam b of round
   it uses seeds[it*num_beams + b]; ICH/PMS: seeds[b] is rank b's srand() seed and its
   rand() stream continues from round to round.  round_best[it] (may be NULL) receives the
   best after round it; best_seq the schedule of the first beam that set the final best. */
int orc_solve_iterations(const orc_instance *inst, int mode, int K, int num_beams, int iterations,
                         const uint32_t *seeds, int32_t initial_bound, int32_t *best,
                         int32_t *best_seq, int32_t *round_best);

/* glibc-compatible rand() stream (restated algorithm), exposed for tests. */
void orc_glibc_rand_fill(uint32_t seed, int32_t *out, int count);

/* gpu-mode hash functions, exposed for tests. */
uint32_t orc_pivot_hash(uint32_t x);
uint32_t orc_noise_hash(uint32_t seed, uint32_t c, uint32_t b);
float orc_gpu_score(int32_t cmax, int32_t num_scheduled, uint32_t seed, uint32_t c, uint32_t b);

/* Verify a schedule (1-based op sequence) and return its makespan, -1 if infeasible. */
int32_t orc_schedule_makespan(const orc_instance *inst, const int32_t *seq);

#ifdef __cplusplus
}
#endif
#endif
