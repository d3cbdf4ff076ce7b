// Test helper: a caller of the C++ drop-in solver entry points written the way the
// reference's drivers call them (gpu/v1/main.cu:50-70, gpu/v1/benchmark.cu:55-65):
// parse_instance into a JSSPInstance, then run_gpu_beam_search_v1 / _v2 with a
// caller-owned out_best_sequence.  It includes only include/bsj_solver.h and links only
// libbsj.so, as a reference driver relinked against this library would.
//
// Reads one case per line from stdin:   v1|v2 <instance file> <K> <best_known> <seed>
// and prints one JSON object per case:  {"makespan": M, "sequence": [...]}
// The sequence buffer is filled with -7 before each call, so a caller can see whether
// the entry point wrote it (it must not when the result is 500000 or more).
//
// With the argument `threads T`, T threads run the whole case list at the same time (the
// entry points serialise on their shared per-device context) and the results are
// printed thread by thread, in case order.
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/bsj_solver.h"

struct Case {
    std::string mode, path;
    int K = 0, best_known = 0, seed = 0;
};

struct Outcome {
    int makespan = 0;
    std::vector<int> sequence;
};

static Outcome run_case(const Case& c, const JSSPInstance& inst)
{
    Outcome o;
    o.sequence.assign((size_t)inst.nbjob * inst.nbmachine, -7);
    if (c.mode == "v1")
        o.makespan = run_gpu_beam_search_v1(inst, c.K, c.best_known, c.seed, o.sequence.data());
    else
        o.makespan = run_gpu_beam_search_v2(inst, c.K, c.best_known, c.seed, o.sequence.data());
    return o;
}

int main(int argc, char** argv)
{
    int threads = 1;
    if (argc == 3 && std::strcmp(argv[1], "threads") == 0) threads = std::atoi(argv[2]);
    if (threads < 1) return 2;
    std::vector<Case> cases;
    char mode[8], path[512];
    int K, bk, seed;
    while (std::scanf("%7s %511s %d %d %d", mode, path, &K, &bk, &seed) == 5)
        cases.push_back(Case{mode, path, K, bk, seed});
    std::vector<JSSPInstance> insts(cases.size());
    for (size_t i = 0; i < cases.size(); i++)
        if (!parse_instance(cases[i].path.c_str(), insts[i])) return 3;

    std::vector<std::vector<Outcome>> out(threads, std::vector<Outcome>(cases.size()));
    auto work = [&](int t) {
        for (size_t i = 0; i < cases.size(); i++) out[t][i] = run_case(cases[i], insts[i]);
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; t++) pool.emplace_back(work, t);
    work(0);
    for (std::thread& th : pool) th.join();

    for (int t = 0; t < threads; t++)
        for (const Outcome& o : out[t]) {
            std::printf("{\"makespan\": %d, \"sequence\": [", o.makespan);
            for (size_t q = 0; q < o.sequence.size(); q++) std::printf("%s%d", q ? ", " : "", o.sequence[q]);
            std::printf("]}\n");
        }
    return 0;
}
