// Driver that runs the reference's own grid selectivity estimate, compiled
// from the reference sources where they lie (see oracle/build_ref.sh).  It
// is test infrastructure: it pins the oracle's restatement of the estimate
// (oracle/pyoracle.py grid_estimate), which the GPU estimate is tested
// against, to the reference's code.
//
// The reference's estimate is spread over three places, none of which
// compiles on its own here, so build_ref.sh copies exactly these lines into
// a temporary build directory outside this repository:
//   * ref_estimate_kernel.inc  - estimateSelectivityKernel
//                                (pierce/query/src/cuda/estimated_overlap.cu:8-41);
//   * ref_estimate_helpers.inc - calculateGlobalAvgSize / calculateGlobalAvgVolRatio
//                                (pierce/query/src/applications/pierce_overlap_main.cpp:189-219);
//   * ref_estimate_pairs.inc   - the estimatePairs lambda of main()
//                                (pierce_overlap_main.cpp:376-471: cell matching,
//                                the kernel's float sum, alpha correction).
// The kernel runs on the host: blockIdx/blockDim/threadIdx are host
// variables and the kernel is called once per matched cell; the reference's
// device-side float reduction (thrust::reduce) becomes a float left fold, and
// sqrtf/powf are the host's, so the raw sum may differ from the GPU's in the
// last bits.
//
// usage: ref_estimate_tool <a.pre> <b.pre> <epsilon> <gamma> <alpha correction 0|1>
//   prints "<raw sum> <estimate> <matched cells>"
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <unordered_map>
#include <vector>

#include "BinaryIO.h"

extern "C" cudaError_t cudaMallocHost(void** ptr, size_t size) {
    *ptr = std::malloc(size ? size : 1);
    return *ptr ? cudaSuccess : cudaErrorMemoryAllocation;
}
extern "C" cudaError_t cudaFreeHost(void* ptr) {
    std::free(ptr);
    return cudaSuccess;
}

namespace {
struct HostDim {
    unsigned x = 0, y = 0, z = 0;
};
HostDim blockIdx, blockDim, threadIdx;
}  // namespace

#undef __global__
#define __global__ static
#include "ref_estimate_kernel.inc"
#undef __global__

#include "ref_estimate_helpers.inc"

namespace {
double g_raw = 0.0;
int g_matched = 0;
}  // namespace

// The reference's host wrapper (estimated_overlap.cu:43-77) copies the
// matched cells to the device, runs the kernel over them and reduces the
// per-cell values in float; the same on the host.
float estimateOverlapSelectivity(const GridCell* a, const GridCell* b, int n, float cellVolume, float epsilon,
                                 float gamma) {
    std::vector<float> out((size_t)std::max(n, 1));
    blockDim.x = 1;
    threadIdx.x = 0;
    for (int i = 0; i < n; ++i) {
        blockIdx.x = (unsigned)i;
        estimateSelectivityKernel(a, b, out.data(), n, cellVolume, epsilon, gamma);
    }
    float total = 0.0f;
    for (int i = 0; i < n; ++i) total += out[i];
    g_raw = total;
    g_matched = n;
    return total;
}

static long long reference_estimate(const GeometryData& mesh1, const GeometryData& mesh2, float epsilon, float gamma,
                                    bool useAlphaCorrection) {
#include "ref_estimate_pairs.inc"
    return estimatePairs(false);
}

int main(int argc, char** argv) {
    if (argc != 6) {
        std::cerr << "usage: ref_estimate_tool <a.pre> <b.pre> <epsilon> <gamma> <alpha 0|1>" << std::endl;
        return 2;
    }
    GeometryData a = RaySpace::IO::readBinaryFile(argv[1]);
    GeometryData b = RaySpace::IO::readBinaryFile(argv[2]);
    if (!a.grid.hasGrid || !b.grid.hasGrid) {
        std::cerr << "inputs need grid statistics" << std::endl;
        return 1;
    }
    const long long est = reference_estimate(a, b, std::strtof(argv[3], nullptr), std::strtof(argv[4], nullptr),
                                             std::atoi(argv[5]) != 0);
    std::printf("%.9g %lld %d\n", g_raw, est, g_matched);
    return 0;
}
