// Driver that runs the reference's own grid statistics, compiled from the
// reference sources where they lie (see oracle/build_ref.sh).  It is test
// infrastructure: it pins this repository's grid statistics (the `.pre`
// producer's --generate-grid) against the reference's generateGridStats.
//
// generateGridStats and the helpers it uses (ObjectStats, Int3Hash,
// Int3Equal: pierce/preprocess/src/pierce_preprocess.cpp:28-167) live in the
// same file as the reference preprocessor's main(), which needs the OBJ
// loader (tinyobjloader, absent); build_ref.sh therefore copies those lines,
// and only those, into a temporary build directory outside this repository
// as ref_grid_stats.inc, which this driver includes.
//
// usage: ref_grid_tool <in.pre> <cell size> <out.pre>
//   reads <in.pre> with RaySpace::IO::readBinaryFile, runs
//   generateGridStats(geometry, geometry.grid, cell size) and writes the
//   result (with its grid) with RaySpace::IO::writeBinaryFile.
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <unordered_map>

#include "BinaryIO.h"

// The reference's pinned allocator calls cudaMallocHost/cudaFreeHost
// (pierce/common/include/PinnedMemory.h:20-46): plain malloc/free here, so
// no CUDA runtime (and no GPU) is needed.
extern "C" cudaError_t cudaMallocHost(void** ptr, size_t size) {
    *ptr = std::malloc(size ? size : 1);
    return *ptr ? cudaSuccess : cudaErrorMemoryAllocation;
}
extern "C" cudaError_t cudaFreeHost(void* ptr) {
    std::free(ptr);
    return cudaSuccess;
}

#include "ref_grid_stats.inc"

int main(int argc, char** argv) {
    if (argc != 4) {
        std::cerr << "usage: ref_grid_tool <in.pre> <cell size> <out.pre>" << std::endl;
        return 2;
    }
    GeometryData g = RaySpace::IO::readBinaryFile(argv[1]);
    if (g.vertices.empty()) {
        std::cerr << "load failed" << std::endl;
        return 1;
    }
    generateGridStats(g, g.grid, std::strtof(argv[2], nullptr));
    return RaySpace::IO::writeBinaryFile(argv[3], g) ? 0 : 1;
}
