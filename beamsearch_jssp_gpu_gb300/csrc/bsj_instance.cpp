// bsj_instance.cpp -- instance files and schedules on the host.
//
// 1. The reference's instance reader as a drop-in (cpu/common/instance_parser.h):
//      bool resolve_instance_file(const char*, char*, int)   instance_parser.cpp:8-34
//      bool parse_instance(const char*, JSSPInstance&)       instance_parser.cpp:37-93
//    exported with the reference's C++ signatures, so a driver that links libbsj.so needs
//    neither instance_parser.cpp nor any other reference source.
// 2. Their C-ABI forms (bsj_instance_resolve / bsj_instance_read) for callers without
//    the C++ types.
// 3. bsj_schedule_decode: the semi-active schedule (start time of every operation) that a
//    dispatch order denotes, with a feasibility check.  The reference returns only the
//    order (gpu/v1/solver.cu:280-284); its start rule is the one applied at every level
//    (gpu/common/gpu_snapshot.cuh:47-70, cpu/common/jssp_types.h:75-97).
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/bsj.h"
#include "../../include/bsj_solver.h"

namespace {

bool readable(const char* path)
{
    FILE* f = std::fopen(path, "r");
    if (!f) return false;
    std::fclose(f);
    return true;
}

// Candidate locations tried after the argument itself, in the reference's order
// (instance_parser.cpp:15-24): Lawrence before Taillard, and Taillard ids without a
// ".txt" suffix.  The list has to match for a bare id to name the same file.
const char* const kSearch[] = {
    "./la%s.txt",
    "./ta%s.txt",
    "./lawrence_instances/la%s.txt",
    "../lawrence_instances/la%s.txt",
    "../../lawrence_instances/la%s.txt",
    "./taillard_instances/ta%s",
    "../taillard_instances/ta%s",
    "../../taillard_instances/ta%s",
};

// Reads the header and up to n*m (machine, duration) pairs the way successive
// fscanf("%d %d") calls do: a pair that cannot be read leaves machine 0 / duration 0,
// and reading stops for good at the first token that is not an integer.
struct TextInstance {
    int n = 0, m = 0;
    std::vector<int> mc, du;  // [n*m], machines 0-based as written in the file
};

enum class ReadResult { Ok, NoFile, NoHeader };

ReadResult read_text(const char* path, TextInstance& t)
{
    FILE* f = std::fopen(path, "r");
    if (!f) return ReadResult::NoFile;
    if (std::fscanf(f, "%d %d", &t.n, &t.m) != 2) {
        std::fclose(f);
        return ReadResult::NoHeader;
    }
    const long long total = (t.n > 0 && t.m > 0) ? (long long)t.n * t.m : 0;
    t.mc.assign((size_t)total, 0);
    t.du.assign((size_t)total, 0);
    bool stuck = false;
    for (long long q = 0; q < total; q++) {
        int a = 0, b = 0;
        if (!stuck) {
            int got = std::fscanf(f, "%d %d", &a, &b);
            if (got < 2) {
                stuck = true;
                if (got < 1) a = 0;
                b = 0;
            }
        }
        t.mc[(size_t)q] = a;
        t.du[(size_t)q] = b;
    }
    std::fclose(f);
    return ReadResult::Ok;
}

}  // namespace

bool resolve_instance_file(const char* input_arg, char* out_path, int path_size)
{
    if (!input_arg || !out_path || path_size < 1) return false;
    std::snprintf(out_path, (size_t)path_size, "%s", input_arg);
    if (readable(out_path)) return true;
    for (const char* fmt : kSearch) {
        std::snprintf(out_path, (size_t)path_size, fmt, input_arg);
        if (readable(out_path)) return true;
    }
    return false;
}

bool parse_instance(const char* filepath, JSSPInstance& inst)
{
    TextInstance t;
    ReadResult r = read_text(filepath, t);
    if (r == ReadResult::NoFile) {
        std::fprintf(stderr, "Error: cannot open instance file: %s\n", filepath);
        return false;
    }
    if (r == ReadResult::NoHeader) {
        std::fprintf(stderr, "Error: cannot read header from %s\n", filepath);
        return false;
    }
    const int n = t.n, m = t.m;
    inst.nbjob = n;
    inst.nbmachine = m;
    inst.nboperation = n * m + 2;
    inst.operations.clear();
    inst.opr_mach.assign((size_t)(m > 0 ? m : 0) + 1, std::vector<int>());
    inst.operations.push_back(Operation{0, 0, 0, 0});
    int id = 1;
    for (int j = 0; j < n; j++) {
        for (int k = 0; k < m; k++, id++) {
            const int mc = t.mc[(size_t)(id - 1)];
            inst.operations.push_back(Operation{id, mc + 1, t.du[(size_t)(id - 1)], j + 1});
            if (mc + 1 >= 0 && mc + 1 <= m) inst.opr_mach[(size_t)(mc + 1)].push_back(id);
        }
    }
    inst.operations.push_back(Operation{n * m + 1, 0, 0, 0});
    return true;
}

extern "C" {

bsj_status bsj_instance_resolve(const char* arg, char* out_path, int32_t path_size)
{
    if (!arg || !out_path || path_size < 1) return BSJ_ERR_INVALID;
    return resolve_instance_file(arg, out_path, path_size) ? BSJ_OK : BSJ_ERR_INVALID;
}

bsj_status bsj_instance_read(const char* path, int32_t* n, int32_t* m, int32_t* machine,
                             int32_t* duration, int32_t capacity)
{
    if (!path || !n || !m) return BSJ_ERR_INVALID;
    TextInstance t;
    if (read_text(path, t) != ReadResult::Ok) return BSJ_ERR_INVALID;
    *n = t.n;
    *m = t.m;
    if (t.n < 1 || t.m < 1) return BSJ_ERR_INVALID;
    if (!machine && !duration) return BSJ_OK;
    if (!machine || !duration) return BSJ_ERR_INVALID;
    if ((long long)t.n * t.m > (long long)capacity) return BSJ_ERR_LIMIT;
    std::memcpy(machine, t.mc.data(), t.mc.size() * sizeof(int32_t));
    std::memcpy(duration, t.du.data(), t.du.size() * sizeof(int32_t));
    return BSJ_OK;
}

bsj_status bsj_schedule_decode(const bsj_instance* inst, const int32_t* sequence, int32_t* start,
                               int32_t* makespan)
{
    if (!inst || !sequence || inst->n < 1 || inst->m < 1 || !inst->machine || !inst->duration)
        return BSJ_ERR_INVALID;
    const int n = inst->n, m = inst->m;
    if ((long long)n * m > (1LL << 26)) return BSJ_ERR_LIMIT;
    std::vector<long long> mready((size_t)m, 0), jready((size_t)n, 0);
    std::vector<int> next((size_t)n, 0);  // next step of each job
    long long cmax = 0;
    for (int q = 0; q < n * m; q++) {
        const int op = sequence[q] - 1;  // 1-based ids: job*m + step + 1
        if (op < 0 || op >= n * m) return BSJ_ERR_INVALID;
        const int j = op / m, k = op % m;
        if (next[(size_t)j] != k) return BSJ_ERR_INVALID;  // repeated op or precedence broken
        const int mc = inst->machine[op], du = inst->duration[op];
        if (mc < 0 || mc >= m || du < 0) return BSJ_ERR_INVALID;
        const long long s = mready[(size_t)mc] > jready[(size_t)j] ? mready[(size_t)mc] : jready[(size_t)j];
        const long long f = s + du;
        if (f > 0x7fffffffLL) return BSJ_ERR_LIMIT;
        mready[(size_t)mc] = f;
        jready[(size_t)j] = f;
        next[(size_t)j] = k + 1;
        if (f > cmax) cmax = f;
        if (start) start[op] = (int32_t)s;
    }
    if (makespan) *makespan = (int32_t)cmax;
    return BSJ_OK;
}

}  // extern "C"
