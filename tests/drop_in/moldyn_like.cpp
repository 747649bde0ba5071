// A driver in the reference's style, built against the compat headers: it
// makes the same IrregularRuntime calls as moldyn/moldyn.cu:311-392 (construct,
// IrregularInit, then per iteration reset_node_data / IrregularStart /
// get_reduction_result / IrregularBarrier) on data read from files.
//
//   moldyn_like <in.bin> <out.bin> <iterations>
// in.bin:  int64 n, int64 e, double param[2] (side, cutoff), double pos[3n],
//          int32 edges[2e]
// out.bin: float forces[3n] after the last iteration (VALUE = float3)
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "include/runtime.h"
#include "irregular/irregular_runtime.h"

struct para {
    double side;
    double cutoffRadius;
};

int main(int argc, char **argv)
{
    if (argc != 4) return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 3;
    int64_t n = 0, e = 0;
    struct para pa;
    if (fread(&n, 8, 1, f) != 1 || fread(&e, 8, 1, f) != 1 || fread(&pa, sizeof(pa), 1, f) != 1)
        return 4;
    std::vector<double> pos(3 * n);
    std::vector<EDGE> edges(e);
    if (fread(pos.data(), sizeof(double), 3 * n, f) != (size_t)(3 * n) ||
        fread(edges.data(), sizeof(EDGE), e, f) != (size_t)e)
        return 5;
    fclose(f);
    int iters = atoi(argv[3]);
    RuntimeInit(argc, argv);
    IrregularRuntime runtime(e, n, edges.data(), NULL, pos.data(), 0, sizeof(double) * 3,
                             sizeof(float) * 3, 3, pos.data(), sizeof(double), &pa,
                             sizeof(struct para), 1, 1);
    runtime.IrregularInit();
    std::vector<float> forces(3 * n);
    for (int it = 0; it < iters; it++) {
        runtime.reset_node_data(pos.data());
        runtime.IrregularStart();
        runtime.get_reduction_result(forces.data());
        runtime.IrregularBarrier();
    }
    RuntimeFinalize();
    FILE *o = fopen(argv[2], "wb");
    if (!o) return 6;
    fwrite(forces.data(), sizeof(float), 3 * n, o);
    fclose(o);
    return 0;
}
