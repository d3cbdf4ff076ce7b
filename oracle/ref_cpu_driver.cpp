// ref_cpu_driver.cpp -- test-only C entry points around the reference CPU solvers.
//
// Linked (by oracle/Makefile, into oracle/_ref/) with the reference's own, unmodified
// sources: cpu/v0_ich/solver.cpp, cpu/v1_pms/solver.cpp and cpu/common/instance_parser.cpp.
// The oracle tests call these to pin the C restatement in bsj_oracle.c and the instance
// parser of the product library.  MPI is not needed: the solvers do not include it; the
// drivers that do (cpu/v1_pms/main.cpp) are replaced by these functions.
#include <cstdlib>
#include <cstring>

#include "jssp_types.h"
#include "instance_parser.h"

// cpu/v0_ich/solver.h:6 and cpu/v1_pms/solver.h:6 (both headers are named solver.h, so
// the two declarations are repeated here instead of included).
int beam_search_ich(const JSSPInstance& inst, int beam_width);
int beam_search_pms(const JSSPInstance& inst, int beam_width, int best_known);

extern "C" {

// srand(seed) then one BS-ICH pass (cpu/v0_ich/main.cpp:39-41 with a chosen seed).
int ref_ich(const char* path, int beam_width, unsigned seed)
{
    JSSPInstance inst;
    if (!parse_instance(path, inst)) return -1;
    srand(seed);
    return beam_search_ich(inst, beam_width);
}

// srand(seed) then one BS-PMS pass (cpu/v1_pms/main.cpp:56,64 for one iteration).
int ref_pms(const char* path, int beam_width, int best_known, unsigned seed)
{
    JSSPInstance inst;
    if (!parse_instance(path, inst)) return -1;
    srand(seed);
    return beam_search_pms(inst, beam_width, best_known);
}

// Several BS-PMS iterations with the bound carried between them, one rank
// (cpu/v1_pms/main.cpp:62-73 with world size 1): returns the final global best.
int ref_pms_iterations(const char* path, int beam_width, unsigned seed, int iterations)
{
    JSSPInstance inst;
    if (!parse_instance(path, inst)) return -1;
    srand(seed);
    int local_best = 500000, global_best = 500000;
    for (int it = 0; it < iterations; it++) {
        int mk = beam_search_pms(inst, beam_width, global_best);
        if (mk < local_best) local_best = mk;
        global_best = local_best;
    }
    return global_best;
}

// Parsed instance, to pin the product parser: fills n, m, nboperation and, for the
// nboperation entries (dummies included), the 1-based machine, duration and job.
int ref_parse(const char* path, int* n, int* m, int* nboperation,
              int* machine1, int* duration, int* job, int capacity)
{
    JSSPInstance inst;
    if (!parse_instance(path, inst)) return -1;
    *n = inst.nbjob;
    *m = inst.nbmachine;
    *nboperation = inst.nboperation;
    int cnt = (int)inst.operations.size();
    if (cnt > capacity) return -2;
    for (int i = 0; i < cnt; i++) {
        machine1[i] = inst.operations[i].num_mc;
        duration[i] = inst.operations[i].dure;
        job[i] = inst.operations[i].num_j;
    }
    return cnt;
}

// Path resolution (cpu/common/instance_parser.cpp:8-34).
int ref_resolve(const char* arg, char* out, int size)
{
    return resolve_instance_file(arg, out, size) ? 1 : 0;
}

}  // extern "C"
