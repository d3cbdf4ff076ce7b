// bsj_cli.cpp -- the reference's command-line drivers, running on the GB300 engine.
//
// One executable under several names; the name it is started by picks the driver:
//   exec_gpu_v1 / exec_gpu_v2              gpu/v1/main.cu:10-84, gpu/v2_twophases/main.cu:10-84
//   exec_gpu_v1_bench / exec_gpu_v2_bench  gpu/v1/benchmark.cu:10-85, gpu/v2_twophases/benchmark.cu
//   BS-ICH                                 cpu/v0_ich/main.cpp:9-55
//   BS-PMS                                 cpu/v1_pms/main.cpp:10-85
//   BS-PMS-bench                           cpu/v1_pms/benchmark.cpp:10-83
//   exec_cpu_time_width (= exec_time_width) cpu/profiling/time_width_study.cpp:11-84
// (or `bsj_cli <name> args...`).  Positional arguments, defaults and printed lines are the
// reference's.  The ICH/PMS drivers run the reference's CPU algorithms as the engine's
// ICH/PMS modes, on the GPU, with identical makespans for identical rand() seeds.
//
// MPI is replaced by beams of one launch: `--ranks R` plays the reference's world size
// (default 1).  Rank r seeds rand() with time(NULL) + r as the reference does, or with
// S + r under `--seed S`, which makes a run repeatable.  Times are wall-clock seconds
// (the reference prints clock(), the CPU time of the process).
//
// Extra options: --device D, --schedule FILE (exec_gpu_*, BS-ICH, BS-PMS: the best
// schedule as CSV job,step,machine,start,finish in dispatch order), and for the suites
// --iters N and --ids a,b,c to shorten them.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "../../include/bsj.h"
#include "../../include/bsj_solver.h"

namespace {

struct Options {
    std::vector<std::string> pos;
    int ranks = 1;
    bool have_seed = false;
    unsigned seed = 0;
    int device = 0;
    std::string schedule;
    int iters = -1;
    std::vector<std::string> ids;
};

bool parse_options(int argc, char** argv, Options& o)
{
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        auto value = [&](const char* name) -> const char* {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "Error: %s needs a value\n", name);
                return nullptr;
            }
            return argv[++i];
        };
        if (a == "--ranks" || a == "--device" || a == "--seed" || a == "--iters" || a == "--schedule" ||
            a == "--ids") {
            const char* v = value(a.c_str());
            if (!v) return false;
            if (a == "--ranks") o.ranks = std::atoi(v);
            else if (a == "--device") o.device = std::atoi(v);
            else if (a == "--seed") { o.seed = (unsigned)std::strtoul(v, nullptr, 10); o.have_seed = true; }
            else if (a == "--iters") o.iters = std::atoi(v);
            else if (a == "--schedule") o.schedule = v;
            else {
                std::string s = v;
                size_t p = 0;
                while (p <= s.size()) {
                    size_t q = s.find(',', p);
                    if (q == std::string::npos) q = s.size();
                    if (q > p) o.ids.push_back(s.substr(p, q - p));
                    p = q + 1;
                }
            }
        } else if (a.size() > 2 && a[0] == '-' && a[1] == '-') {
            std::fprintf(stderr, "Error: unknown option %s\n", a.c_str());
            return false;
        } else {
            o.pos.push_back(a);
        }
    }
    if (o.ranks < 1) {
        std::fprintf(stderr, "Error: --ranks must be >= 1\n");
        return false;
    }
    return true;
}

unsigned seed_base(const Options& o) { return o.have_seed ? o.seed : (unsigned)std::time(nullptr); }

double seconds_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// The engine's 0-based arrays from the reference's instance type.
struct Arrays {
    std::vector<int32_t> mc, du;
    bsj_instance view() const
    {
        return bsj_instance{n, m, mc.data(), du.data()};
    }
    int n = 0, m = 0;
};

Arrays to_arrays(const JSSPInstance& inst)
{
    Arrays a;
    a.n = inst.nbjob;
    a.m = inst.nbmachine;
    const int N = a.n * a.m;
    a.mc.resize((size_t)N);
    a.du.resize((size_t)N);
    for (int q = 0; q < N; q++) {
        a.mc[(size_t)q] = inst.operations[(size_t)q + 1].num_mc - 1;
        a.du[(size_t)q] = inst.operations[(size_t)q + 1].dure;
    }
    return a;
}

struct Engine {
    bsj_context* ctx = nullptr;
    explicit Engine(int device)
    {
        if (bsj_create(&ctx, device) != BSJ_OK) {
            std::fprintf(stderr, "Error: cannot open CUDA device %d\n", device);
            std::exit(EXIT_FAILURE);
        }
    }
    ~Engine() { bsj_destroy(ctx); }
    void check(bsj_status s) const
    {
        if (s != BSJ_OK) {
            std::fprintf(stderr, "Error: %s: %s\n", bsj_status_string(s), bsj_last_error(ctx));
            std::exit(EXIT_FAILURE);
        }
    }
};

// Multi-start run: `iterations` rounds of `ranks` beams with the bound carried (the MPI loop
// of every driver).  Gpu modes: rank r's round seeds are its successive rand() draws after
// srand(base + r).  ICH/PMS: rank r's stream is srand(base + r), continued across rounds.
struct RunResult {
    int32_t best = BSJ_NO_BOUND;
    std::vector<int32_t> seq;
    std::vector<int32_t> rounds;
};

RunResult run_ranks(Engine& eng, const Arrays& a, int mode, int K, int ranks, int iterations, unsigned base)
{
    const bool carry = (mode == BSJ_MODE_ICH || mode == BSJ_MODE_PMS);
    std::vector<uint32_t> seeds;
    if (carry) {
        for (int r = 0; r < ranks; r++) seeds.push_back(base + (unsigned)r);
    } else {
        seeds.assign((size_t)iterations * ranks, 0);
        for (int r = 0; r < ranks; r++) {
            std::srand(base + (unsigned)r);
            for (int it = 0; it < iterations; it++) seeds[(size_t)it * ranks + r] = (uint32_t)std::rand();
        }
    }
    RunResult out;
    out.seq.assign((size_t)a.n * a.m, 0);
    out.rounds.assign((size_t)iterations, 0);
    const bsj_instance inst = a.view();
    eng.check(bsj_solve_iterations(eng.ctx, &inst, mode, K, ranks, iterations, seeds.data(), BSJ_NO_BOUND,
                                   &out.best, out.seq.data(), out.rounds.data(), nullptr));
    return out;
}

void write_schedule(const std::string& path, const Arrays& a, const std::vector<int32_t>& seq)
{
    std::vector<int32_t> start((size_t)a.n * a.m, 0);
    int32_t cmax = 0;
    const bsj_instance inst = a.view();
    if (bsj_schedule_decode(&inst, seq.data(), start.data(), &cmax) != BSJ_OK) {
        std::fprintf(stderr, "Error: no complete schedule to write\n");
        return;
    }
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) {
        std::fprintf(stderr, "Error: cannot write %s\n", path.c_str());
        return;
    }
    std::fprintf(f, "job,step,machine,start,finish\n");
    for (int32_t id : seq) {
        const int op = id - 1, j = op / a.m, k = op % a.m;
        std::fprintf(f, "%d,%d,%d,%d,%d\n", j + 1, k + 1, a.mc[(size_t)op] + 1, start[(size_t)op],
                     start[(size_t)op] + a.du[(size_t)op]);
    }
    std::fclose(f);
}

int device_count()
{
    int32_t c = 0;
    return bsj_device_count(&c) == BSJ_OK ? c : 0;
}

// ---- exec_gpu_v1 / exec_gpu_v2 (gpu/v1/main.cu, gpu/v2_twophases/main.cu) ----
int main_gpu(const Options& o, int mode)
{
    char file[512] = "./la33.txt";
    int K = (mode == BSJ_MODE_V1) ? 1000 : 5000;
    int iterations = 100;
    if (o.pos.size() > 0 && !resolve_instance_file(o.pos[0].c_str(), file, sizeof(file))) {
        std::fprintf(stderr, "Error: cannot locate instance file: %s\n", o.pos[0].c_str());
        return 1;
    }
    if (o.pos.size() > 1) K = std::atoi(o.pos[1].c_str());
    if (o.pos.size() > 2) iterations = std::atoi(o.pos[2].c_str());
    JSSPInstance inst;
    if (!parse_instance(file, inst)) return 1;
    const bool v1 = (mode == BSJ_MODE_V1);
    const char* rule = v1 ? "============================" : "=======================================";
    std::printf(v1 ? "=== GPU Beam Search (v1) ===\n" : "=== GPU Beam Search (v2 Two-Phases) ===\n");
    std::printf("Instance: %s  |  Jobs: %d  |  Machines: %d\n", file, inst.nbjob, inst.nbmachine);
    std::printf("Beam Width (K): %d  |  MPI Ranks: %d  |  GPUs/Node: %d  |  Iterations: %d\n", K, o.ranks,
                device_count(), iterations);
    std::printf("%s\n", rule);
    std::fflush(stdout);
    if (K < 1 || iterations < 1) {
        std::fprintf(stderr, "Error: beam width and iterations must be >= 1\n");
        return 1;
    }
    Engine eng(o.device);
    const Arrays a = to_arrays(inst);
    auto t0 = std::chrono::steady_clock::now();
    RunResult r = run_ranks(eng, a, mode, K, o.ranks, iterations, seed_base(o));
    const double el = seconds_since(t0);
    std::printf("%s\n", rule);
    std::printf("Best Makespan  : %d\n", r.best);
    std::printf("Execution Time : %.2f seconds\n", el);
    if (!o.schedule.empty()) write_schedule(o.schedule, a, r.seq);
    return 0;
}

const char* const kLawrence[] = {"01", "02", "03", "04", "05", "06", "07", "08", "09", "10",
                                 "11", "12", "13", "14", "15", "16", "17", "18", "19", "20",
                                 "21", "22", "23", "24", "25", "26", "27", "28", "29", "30",
                                 "31", "32", "33", "34", "35", "36", "37", "38", "39", "40"};

void table_header(const char* first)
{
    std::printf("\n%-8s %-30s %-6s %-9s %-8s %-12s %-10s\n", first, "Instance", "Jobs", "Machines", "Ops",
                "BestSpan", "Time(s)");
    std::printf("-------------------------------------------------------------------------------\n");
}

void table_row(int K, const char* path, const JSSPInstance& inst, int best, double el)
{
    std::printf("%-8d %-30s %-6d %-9d %-8d %-12d %-10.2f\n", K, path, inst.nbjob, inst.nbmachine,
                inst.nboperation, best, el);
    std::fflush(stdout);
}

// ---- suites: exec_gpu_v*_bench (gpu/v1/benchmark.cu), BS-PMS-bench (cpu/v1_pms/benchmark.cpp) ----
int main_suite(const Options& o, int mode, int default_iters, const char* done_line)
{
    table_header("Kbest");
    std::vector<std::string> ids;
    if (o.ids.empty()) ids.assign(std::begin(kLawrence), std::end(kLawrence));
    else ids = o.ids;
    const int iterations = o.iters > 0 ? o.iters : default_iters;
    Engine eng(o.device);
    for (size_t idx = 0; idx < ids.size(); idx++) {
        char path[512];
        if (!resolve_instance_file(ids[idx].c_str(), path, sizeof(path))) {
            std::printf("SKIP la%s  (file not found)\n", ids[idx].c_str());
            continue;
        }
        JSSPInstance inst;
        if (!parse_instance(path, inst)) continue;
        // the reference's widths: 1000 for its first ten ids, 5000 afterwards
        int pos = 0;
        for (; pos < 40 && ids[idx] != kLawrence[pos]; pos++) {}
        const int K = (pos < 10) ? 1000 : 5000;
        const Arrays a = to_arrays(inst);
        auto t0 = std::chrono::steady_clock::now();
        RunResult r = run_ranks(eng, a, mode, K, o.ranks, iterations, seed_base(o));
        table_row(K, path, inst, r.best, seconds_since(t0));
    }
    std::printf("\n%s\n", done_line);
    return 0;
}

// ---- BS-ICH (cpu/v0_ich/main.cpp) ----
int main_ich(const Options& o)
{
    char file[512] = "./la33.txt";
    int K = 5000;
    JSSPInstance inst;
    if (o.pos.size() > 0) {
        if (!resolve_instance_file(o.pos[0].c_str(), file, sizeof(file))) {
            std::fprintf(stderr, "Error: cannot locate instance file for: %s\n", o.pos[0].c_str());
            return 1;
        }
    }
    if (o.pos.size() > 1) {
        K = std::atoi(o.pos[1].c_str());
        if (K < 1) {
            std::fprintf(stderr, "Error: beam_width must be >= 1\n");
            return 1;
        }
    }
    if (!parse_instance(file, inst)) return 1;
    std::printf("  Instance File : %s\n", file);
    std::printf("  Jobs          : %d\n", inst.nbjob);
    std::printf("  Machines      : %d\n", inst.nbmachine);
    std::printf("  Beam Width (K): %d\n", K);
    std::fflush(stdout);
    Engine eng(o.device);
    const Arrays a = to_arrays(inst);
    auto t0 = std::chrono::steady_clock::now();
    // srand(12345) then one pass (cpu/v0_ich/main.cpp:39-41); --seed replaces 12345
    RunResult r = run_ranks(eng, a, BSJ_MODE_ICH, K, 1, 1, o.have_seed ? o.seed : 12345u);
    const double el = seconds_since(t0);
    std::printf("  ===========================\n");
    std::printf("  Scheduled Ops    : %d\n", inst.nbjob * inst.nbmachine);
    std::printf("  Best Makespan    : %d\n", r.best);
    std::printf("  Execution Time   : %g seconds\n", el);
    if (!o.schedule.empty()) write_schedule(o.schedule, a, r.seq);
    return 0;
}

// ---- BS-PMS (cpu/v1_pms/main.cpp) ----
int main_pms(const Options& o)
{
    char file[512] = "./la33.txt";
    int K = 5000;
    const int iterations = o.iters > 0 ? o.iters : 100;
    JSSPInstance inst;
    if (o.pos.size() > 0) {
        if (!resolve_instance_file(o.pos[0].c_str(), file, sizeof(file))) {
            std::fprintf(stderr, "Error: cannot locate instance file for: %s\n", o.pos[0].c_str());
            return 1;
        }
    }
    if (o.pos.size() > 1) {
        K = std::atoi(o.pos[1].c_str());
        if (K < 1) {
            std::fprintf(stderr, "Error: beam_width must be >= 1\n");
            return 1;
        }
    }
    if (!parse_instance(file, inst)) return 1;
    std::printf("  Instance : %s  (%d jobs x %d machines)\n", file, inst.nbjob, inst.nbmachine);
    std::printf("  Beam     : %d  |  Ranks : %d  |  Iterations : %d\n", K, o.ranks, iterations);
    std::fflush(stdout);
    Engine eng(o.device);
    const Arrays a = to_arrays(inst);
    auto t0 = std::chrono::steady_clock::now();
    RunResult r = run_ranks(eng, a, BSJ_MODE_PMS, K, o.ranks, iterations, seed_base(o));
    const double el = seconds_since(t0);
    for (int it = 0; it < iterations; it += 10) std::printf("  iter %4d | global best = %d\n", it, r.rounds[(size_t)it]);
    std::printf("  ===========================\n");
    std::printf("  Best Makespan  : %d\n", r.best);
    std::printf("  Execution Time : %.2f seconds\n", el);
    if (!o.schedule.empty()) write_schedule(o.schedule, a, r.seq);
    return 0;
}

// ---- exec_time_width (cpu/profiling/time_width_study.cpp): BS-PMS time vs beam width ----
int main_time_width(const Options& o)
{
    std::vector<std::string> ids = o.ids.empty() ? std::vector<std::string>{"10", "15", "21", "31"} : o.ids;
    const int widths[] = {100, 200, 400, 800, 1600, 3200, 6400, 12800, 25600};
    const int iterations = o.iters > 0 ? o.iters : 100;
    table_header("Width");
    Engine eng(o.device);
    const unsigned base = seed_base(o);
    for (const std::string& id : ids) {
        char path[512];
        if (!resolve_instance_file(id.c_str(), path, sizeof(path))) {
            std::printf("SKIP la%s (file not found)\n", id.c_str());
            continue;
        }
        JSSPInstance inst;
        if (!parse_instance(path, inst)) continue;
        std::printf("\n==== Instance %s ====\n", path);
        const Arrays a = to_arrays(inst);
        for (size_t w = 0; w < sizeof(widths) / sizeof(widths[0]); w++) {
            const int K = widths[w];
            if (K > BSJ_MAX_BEAM) {
                std::printf("%-8d %-30s width above the engine's limit (%d)\n", K, path, BSJ_MAX_BEAM);
                continue;
            }
            // srand(time + rank + w) per width (time_width_study.cpp:52)
            auto t0 = std::chrono::steady_clock::now();
            RunResult r = run_ranks(eng, a, BSJ_MODE_PMS, K, o.ranks, iterations, base + (unsigned)w);
            table_row(K, path, inst, r.best, seconds_since(t0));
        }
    }
    std::printf("\nTime vs Beam Width study finished.\n");
    return 0;
}

std::string base_name(const char* p)
{
    std::string s = p ? p : "";
    size_t k = s.find_last_of('/');
    return k == std::string::npos ? s : s.substr(k + 1);
}

}  // namespace

int main(int argc, char** argv)
{
    std::string tool = base_name(argv[0]);
    int shift = 0;
    if (tool == "bsj_cli") {
        if (argc < 2) {
            std::fprintf(stderr,
                         "usage: bsj_cli <exec_gpu_v1|exec_gpu_v2|exec_gpu_v1_bench|exec_gpu_v2_bench|"
                         "BS-ICH|BS-PMS|BS-PMS-bench|exec_cpu_time_width> [args]\n");
            return 2;
        }
        tool = argv[1];
        shift = 1;
    }
    Options o;
    if (!parse_options(argc - shift, argv + shift, o)) return 1;
    if (tool == "exec_gpu_v1") return main_gpu(o, BSJ_MODE_V1);
    if (tool == "exec_gpu_v2") return main_gpu(o, BSJ_MODE_V2);
    if (tool == "exec_gpu_v1_bench") return main_suite(o, BSJ_MODE_V1, 50, "All Lawrence instances finished.");
    if (tool == "exec_gpu_v2_bench") return main_suite(o, BSJ_MODE_V2, 50, "All Lawrence instances finished.");
    if (tool == "BS-ICH") return main_ich(o);
    if (tool == "BS-PMS") return main_pms(o);
    if (tool == "BS-PMS-bench") return main_suite(o, BSJ_MODE_PMS, 100, "All instances finished.");
    if (tool == "exec_cpu_time_width" || tool == "exec_time_width") return main_time_width(o);
    std::fprintf(stderr, "bsj_cli: unknown driver name '%s'\n", tool.c_str());
    return 2;
}
