// Writes the reference's model constants for its GPU kernel: the 72 NUM_POS
// floats that time_GPU.cu:117-120 fills with initTransforms and
// initInertiaTensors (helpers_CPU/dynamicsGradient.h:124-212, :487-587) and
// uploads as d_mem_const (:174).  Compiled UNMODIFIED from the reference tree
// behind oracle/eigen_shim; run at build time where that tree is present, so
// the binary file oracle/_ref/ref_const.bin travels with the cubin of
// oracle/ref_gpu_kernels.cu.
//
// ORACLE TEST INFRASTRUCTURE ONLY.
#include <cstdio>
#include "utils/ReusableThreads.h"
#include "helpers_CPU/dynamicsGradient.h"

int main(int argc, char **argv) {
    if (argc != 2) {
        std::fprintf(stderr, "usage: %s out.bin\n", argv[0]);
        return 2;
    }
    static float c[72 * NUM_POS];
    initTransforms(c);
    initInertiaTensors(c + 36 * NUM_POS);
    std::FILE *f = std::fopen(argv[1], "wb");
    if (!f || std::fwrite(c, sizeof(float), 72 * NUM_POS, f) != 72 * NUM_POS || std::fclose(f) != 0) {
        std::perror(argv[1]);
        return 1;
    }
    return 0;
}
