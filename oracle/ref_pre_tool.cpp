// Driver that runs the reference's own `.pre` reader, edge extractor and
// writer, compiled from the reference sources where they lie (see
// oracle/build_ref.sh).  It is test infrastructure: it pins this repository's
// `.pre` writer and edge extractor byte-for-byte against the reference
// (pierce/common/include/BinaryIO.h, pierce/preprocess/src/EdgePreprocessor.cpp).
//
// usage: ref_pre_tool <in.pre> <out.pre>
//   reads <in.pre> with RaySpace::IO::readBinaryFile, replaces its edge
//   payload by EdgePreprocessor::extractEdges(indices, triangleToObject,
//   vertices) and writes the result with RaySpace::IO::writeBinaryFile.
//
// The reference keeps geometry in std::vectors whose allocator calls
// cudaMallocHost/cudaFreeHost (pierce/common/include/PinnedMemory.h:20-46);
// on a host without a GPU those calls fail, so this driver defines both
// symbols itself as plain malloc/free and is linked without the CUDA runtime.
#include <cstdlib>
#include <cstring>
#include <iostream>

#include "BinaryIO.h"
#include "EdgePreprocessor.h"

extern "C" cudaError_t cudaMallocHost(void** ptr, size_t size) {
    *ptr = std::malloc(size ? size : 1);
    return *ptr ? cudaSuccess : cudaErrorMemoryAllocation;
}
extern "C" cudaError_t cudaFreeHost(void* ptr) {
    std::free(ptr);
    return cudaSuccess;
}

int main(int argc, char** argv) {
    if (argc != 3) {
        std::cerr << "usage: ref_pre_tool <in.pre> <out.pre>" << std::endl;
        return 2;
    }
    GeometryData g = RaySpace::IO::readBinaryFile(argv[1]);
    if (g.vertices.empty()) {
        std::cerr << "load failed" << std::endl;
        return 1;
    }
    g.edges = EdgePreprocessor::extractEdges(g.indices, g.triangleToObject, g.vertices);
    if (!RaySpace::IO::writeBinaryFile(argv[2], g)) return 1;
    std::cout << "edges " << g.edges.numEdges() << std::endl;
    return 0;
}
