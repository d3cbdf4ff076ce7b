// Test helper: parses an instance with the library's C++ drop-in parse_instance /
// resolve_instance_file (include/bsj_solver.h) and prints what it read, one line per
// field, so a test can compare it with the reference parser's result.
#include <cstdio>

#include "../../include/bsj_solver.h"

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    char path[512];
    if (!resolve_instance_file(argv[1], path, sizeof(path))) {
        std::printf("unresolved\n");
        return 3;
    }
    std::printf("path %s\n", path);
    JSSPInstance inst;
    if (!parse_instance(path, inst)) {
        std::printf("unparsed\n");
        return 4;
    }
    std::printf("n %d\nm %d\nnboperation %d\n", inst.nbjob, inst.nbmachine, inst.nboperation);
    std::printf("machine1");
    for (const Operation& op : inst.operations) std::printf(" %d", op.num_mc);
    std::printf("\nduration");
    for (const Operation& op : inst.operations) std::printf(" %d", op.dure);
    std::printf("\njob");
    for (const Operation& op : inst.operations) std::printf(" %d", op.num_j);
    std::printf("\nid");
    for (const Operation& op : inst.operations) std::printf(" %d", op.num_op);
    std::printf("\n");
    return 0;
}
