// Radix sort, scan and unique: library calls into CUB (part of the CUDA
// toolkit), used by the BVH build (Morton sort), the two-pass join (count
// scan) and pair de-duplication.  They replace the reference's Thrust calls
// (pierce/query/src/cuda/scan_utils.cu:11-28,
//  pierce/query/src/cuda/mesh_query_deduplication.cu:56-90).
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/iterator/transform_iterator.h>

#include "common.cuh"

namespace pgpu {

namespace {
struct ToI64 {
    __host__ __device__ int64_t operator()(int32_t v) const { return (int64_t)v; }
};
}  // namespace

int sort_u32_pairs(pierce_ctx* ctx, uint32_t* keys_in, uint32_t* keys_out, uint32_t* vals_in, uint32_t* vals_out,
                   int64_t n, int end_bit) {
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, keys_in, keys_out, vals_in, vals_out, n, 0, end_bit,
                                    ctx->stream);
    void* tmp = nullptr;
    if (int s = scratch(ctx, 0, bytes, &tmp)) return s;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(tmp, bytes, keys_in, keys_out, vals_in, vals_out, n, 0, end_bit,
                                                    ctx->stream);
    ctx->launches += 4;
    return check_cuda(e, "radix sort (pairs)");
}

int sort_u64_pairs(pierce_ctx* ctx, uint64_t* keys_in, uint64_t* keys_out, uint32_t* vals_in, uint32_t* vals_out,
                   int64_t n, int end_bit) {
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, keys_in, keys_out, vals_in, vals_out, n, 0, end_bit,
                                    ctx->stream);
    void* tmp = nullptr;
    if (int s = scratch(ctx, 0, bytes, &tmp)) return s;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(tmp, bytes, keys_in, keys_out, vals_in, vals_out, n, 0, end_bit,
                                                    ctx->stream);
    ctx->launches += (end_bit + 7) / 8;
    return check_cuda(e, "radix sort (64-bit pairs)");
}

int sort_u64_keys(pierce_ctx* ctx, uint64_t* keys_in, uint64_t* keys_out, int64_t n) {
    size_t bytes = 0;
    cub::DeviceRadixSort::SortKeys(nullptr, bytes, keys_in, keys_out, n, 0, 64, ctx->stream);
    void* tmp = nullptr;
    if (int s = scratch(ctx, 0, bytes, &tmp)) return s;
    cudaError_t e = cub::DeviceRadixSort::SortKeys(tmp, bytes, keys_in, keys_out, n, 0, 64, ctx->stream);
    ctx->launches += 8;
    return check_cuda(e, "radix sort (keys)");
}

int exclusive_scan_i32_to_i64(pierce_ctx* ctx, const int32_t* in, int64_t* out, int64_t n) {
    auto it = thrust::make_transform_iterator(in, ToI64());
    size_t bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, bytes, it, out, n, ctx->stream);
    void* tmp = nullptr;
    if (int s = scratch(ctx, 0, bytes, &tmp)) return s;
    cudaError_t e = cub::DeviceScan::ExclusiveSum(tmp, bytes, it, out, n, ctx->stream);
    ctx->launches += 2;
    return check_cuda(e, "exclusive scan");
}

int exclusive_scan_i32(pierce_ctx* ctx, const int32_t* in, int32_t* out, int64_t n) {
    size_t bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, n, ctx->stream);
    void* tmp = nullptr;
    if (int s = scratch(ctx, 0, bytes, &tmp)) return s;
    cudaError_t e = cub::DeviceScan::ExclusiveSum(tmp, bytes, in, out, n, ctx->stream);
    ctx->launches += 2;
    return check_cuda(e, "exclusive scan (int32)");
}

// Indices i < n with flags[i] != 0, in increasing order, into out; the count
// stays on the device (*d_count, 64-bit).  Order-preserving, so lists built
// from it (and the hierarchies built over them) do not depend on scheduling.
int select_flagged(pierce_ctx* ctx, const uint8_t* flags, int64_t n, uint32_t* out, unsigned long long* d_count) {
    thrust::counting_iterator<uint32_t> ids(0);
    size_t bytes = 0;
    cub::DeviceSelect::Flagged(nullptr, bytes, ids, flags, out, d_count, n, ctx->stream);
    void* tmp = nullptr;
    if (int s = scratch(ctx, 0, bytes, &tmp)) return s;
    cudaError_t e = cub::DeviceSelect::Flagged(tmp, bytes, ids, flags, out, d_count, n, ctx->stream);
    ctx->launches += 2;
    return check_cuda(e, "select flagged");
}

// Unique of a sorted key array; the count is read back synchronously.
int unique_u64(pierce_ctx* ctx, const uint64_t* in, uint64_t* out, int64_t n, int64_t* num_unique) {
    // the selected-count word lives right after the CUB temp storage in scratch slot 0
    size_t bytes = 0;
    void* pcount = nullptr;
    cub::DeviceSelect::Unique(nullptr, bytes, in, out, (int64_t*)nullptr, n, ctx->stream);
    const size_t aligned = (bytes + 255) & ~(size_t)255;
    void* tmp = nullptr;
    if (int s = scratch(ctx, 0, aligned + 256, &tmp)) return s;
    pcount = static_cast<char*>(tmp) + aligned;
    cudaError_t e = cub::DeviceSelect::Unique(tmp, bytes, in, out, static_cast<int64_t*>(pcount), n, ctx->stream);
    ctx->launches += 2;
    if (int s = check_cuda(e, "unique")) return s;
    return host_value(ctx, pcount, 8, num_unique, "unique count");
}

}  // namespace pgpu
