/*
 * ref_multi_tables.cpp - prints the face tables of the reference's multi-GPU
 * program, produced by running its own getLaplacian and getPositions
 * (koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC_multi.cu:73-271).
 *
 * Test infrastructure only.  Linked by oracle/Makefile against that file's host
 * code where it lies; the binary is written to oracle/_ref/ and run by
 * tests/golden/make_golden.py, which commits what it prints as
 * tests/golden/ref_multi_tables.json.  Nothing here is shipped.
 *
 * Per face f = 4 * slot + k: the neighbour's block offset (blockDirs), its slot
 * (valueInds) and the Hodge weight before scaling (hodges).
 */
#include <cuda_runtime.h>
#include <cstdio>

#include "jukan_koodit/Types/Buffer.hpp"
#include "jukan_koodit/Types/Vector3.hpp"

// Defined in GPUGrossPitaevskii_BCC_multi.cu.
void getPositions(Buffer<Vector3> &pos);
ddouble getLaplacian(Buffer<int3> &blockDirs, Buffer<int> &valueInds, Buffer<ddouble> &hodges);

int main()
{
    Buffer<Vector3> pos;
    getPositions(pos);
    Buffer<int3> dirs;
    Buffer<int> slots;
    Buffer<ddouble> hodges;
    const ddouble ret = getLaplacian(dirs, slots, hodges);
    std::printf("{\n  \"source\": \"koodit/GrossPitaevskii/GPUGrossPitaevskii_BCC_multi.cu:73-271\",\n");
    std::printf("  \"returned_hodge\": %.17g,\n  \"faces\": [\n", ret);
    for (unsigned f = 0; f < dirs.size(); f++)
        std::printf("    [%d, %d, %d, %d, %.17g]%s\n", dirs[f].x, dirs[f].y, dirs[f].z, slots[f], hodges[f],
                    f + 1 < dirs.size() ? "," : "");
    std::printf("  ],\n  \"positions\": [\n");
    for (unsigned l = 0; l < pos.size(); l++)
        std::printf("    [%.17g, %.17g, %.17g]%s\n", pos[l].x, pos[l].y, pos[l].z, l + 1 < pos.size() ? "," : "");
    std::printf("  ]\n}\n");
    return 0;
}
