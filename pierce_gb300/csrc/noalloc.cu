// Pair de-duplication that allocates nothing.
//
// Some callers of this library cannot allocate device memory at the point
// where they need de-duplicated pairs: code running inside a host callback
// or between stream-ordered steps that must not synchronise the device
// (cudaMalloc and cudaFree synchronise), plug-ins that run under a memory
// budget owned by their host application, and allocators that forbid
// foreign allocations on their pool.  pierce_deduplicate_pairs_noalloc
// gives them the de-duplication of pierce_merge_and_deduplicate_pairs with
// its scratch memory taken from a fixed array that the library declares in
// this file; the caller provides the input and output buffers.
//
// Scratch: one open-addressing hash set of PIERCE_NOALLOC_TABLE_SLOTS
// 64-bit keys (32 MiB) plus a few control words, a file-scope __device__
// array.  Every GPU that loads this library holds that array until the
// process exits.  At most PIERCE_NOALLOC_MAX_PAIRS input pairs are accepted,
// which keeps the load factor at or below 1/2 so that no insert can run out
// of slots.
//
// The array starts zeroed when the module loads (zero is a valid key, the
// pair (0, 0)), so the first call on a device -- and the first call after a
// device reset reloads the module -- clears it; the array itself records
// that it was cleared (kWordReady), so no host-side state can go stale.
// After that every call leaves the table empty: compaction resets each slot
// it reads.  The pair (-1, -1) packs to the empty-slot marker, so it is
// recorded in a flag word (kWordMarker) and appended by the compaction.
#include <cuda_runtime.h>

#include <cstdio>

#include "common.cuh"

namespace {

constexpr uint64_t kTableSlots = PIERCE_NOALLOC_TABLE_SLOTS;
constexpr uint64_t kWordReady = kTableSlots;       // kReadyMagic once the table is cleared
constexpr uint64_t kWordMarker = kTableSlots + 1;  // 1: the pair (-1, -1) was among the inputs
constexpr uint64_t kArrayWords = kTableSlots + 32;
constexpr unsigned long long kReadyMagic = 0x5049455243453031ull;
constexpr unsigned long long kEmpty = 0xFFFFFFFFFFFFFFFFull;

// The scratch array.  Host code must not pass this symbol to a kernel: on
// the host it names a stand-in, not the device address; the address comes
// from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned long long g_noalloc_table[kArrayWords];

__device__ __forceinline__ unsigned long long mix(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

// Clears the table unless it is already marked as cleared.
__global__ void k_noalloc_prepare(unsigned long long* table) {
    if (__ldcg(table + kWordReady) == kReadyMagic) return;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < kTableSlots;
         i += (uint64_t)gridDim.x * blockDim.x)
        table[i] = kEmpty;
    if (blockIdx.x == 0 && threadIdx.x == 0) table[kWordMarker] = 0;
}

__global__ void k_noalloc_mark_ready(unsigned long long* table) { table[kWordReady] = kReadyMagic; }

__global__ void k_noalloc_insert(const uint64_t* __restrict__ pairs, int64_t n, unsigned long long* table) {
    const unsigned long long mask = kTableSlots - 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t v = pairs[i];                       // pierce_pair {a, b} as a 64-bit word
        const unsigned long long key = (v >> 32) | (v << 32);  // (a << 32) | b
        if (key == kEmpty) {  // the pair (-1, -1)
            table[kWordMarker] = 1;
            continue;
        }
        unsigned long long h = mix(key) & mask;
        // Load factor <= 1/2 is guaranteed by the size check, so an empty
        // slot is always reached; the bound only makes the loop finite.
        for (unsigned long long probe = 0; probe < kTableSlots; ++probe) {
            const unsigned long long cur = __ldcg(table + h);
            if (cur == key) break;
            if (cur == kEmpty) {
                const unsigned long long old = atomicCAS(table + h, kEmpty, key);
                if (old == kEmpty || old == key) break;
            }
            h = (h + 1) & mask;
        }
    }
}

// Occupied slots -> out (warp-aggregated cursor); each slot read is reset to
// empty, so the table is empty again for the next call.
__global__ void k_noalloc_compact(unsigned long long* __restrict__ table, uint64_t* __restrict__ out,
                                  unsigned long long* count) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && table[kWordMarker]) {
        table[kWordMarker] = 0;
        out[atomicAdd(count, 1ull)] = kEmpty;  // the pair (-1, -1)
    }
    for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x; base < kTableSlots;
         base += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = base + threadIdx.x;
        const unsigned long long key = i < kTableSlots ? table[i] : kEmpty;
        const bool valid = key != kEmpty;
        if (valid) table[i] = kEmpty;
        const unsigned ballot = __ballot_sync(0xFFFFFFFFu, valid);
        if (!ballot) continue;
        const int lane = threadIdx.x & 31;
        unsigned long long wbase = 0;
        if (lane == 0) wbase = atomicAdd(count, (unsigned long long)__popc(ballot));
        wbase = __shfl_sync(0xFFFFFFFFu, wbase, 0);
        if (valid) out[wbase + __popc(ballot & ((1u << lane) - 1u))] = (key >> 32) | (key << 32);
    }
}

// Device address of the scratch array on the current device, looked up on
// every call (it allocates nothing and stays right after a device reset).
int table_address(void** out) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_table);
    if (e != cudaSuccess || ptr == nullptr) {
        cudaGetLastError();
        char msg[256];
        std::snprintf(msg, sizeof(msg), "deduplicate_pairs_noalloc: cudaGetSymbolAddress failed: %s",
                      cudaGetErrorString(e));
        return pgpu::set_error_cstr(PIERCE_ERR_CUDA, msg);
    }
    *out = ptr;
    return PIERCE_OK;
}

}  // namespace

extern "C" int pierce_deduplicate_pairs_noalloc(const pierce_pair* d_pairs, int64_t n, pierce_pair* d_out,
                                                uint64_t* d_num_unique, void* stream) {
    if (n < 0 || (n > 0 && (!d_pairs || !d_out)) || !d_num_unique)
        return pgpu::set_error_cstr(PIERCE_ERR_INVALID_ARGUMENT, "deduplicate_pairs_noalloc: null pointer or n < 0");
    if ((uint64_t)n > (uint64_t)PIERCE_NOALLOC_MAX_PAIRS) {
        char msg[200];
        std::snprintf(msg, sizeof(msg),
                      "deduplicate_pairs_noalloc: %lld input pairs exceed the maximum of %lld "
                      "(use pierce_merge_and_deduplicate_pairs for larger inputs)",
                      (long long)n, (long long)PIERCE_NOALLOC_MAX_PAIRS);
        return pgpu::set_error_cstr(PIERCE_ERR_INVALID_ARGUMENT, msg);
    }
    void* table = nullptr;
    if (int s = table_address(&table)) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned long long* tab = static_cast<unsigned long long*>(table);
    cudaError_t e = cudaMemsetAsync(d_num_unique, 0, sizeof(uint64_t), st);
    if (e == cudaSuccess && n > 0) {
        const int block = 256;
        const int grid = (int)((n + block - 1) / block < 4096 ? (n + block - 1) / block : 4096);
        k_noalloc_prepare<<<1024, 256, 0, st>>>(tab);
        k_noalloc_mark_ready<<<1, 1, 0, st>>>(tab);
        k_noalloc_insert<<<grid, block, 0, st>>>(reinterpret_cast<const uint64_t*>(d_pairs), n, tab);
        k_noalloc_compact<<<4096, 256, 0, st>>>(tab, reinterpret_cast<uint64_t*>(d_out),
                                                reinterpret_cast<unsigned long long*>(d_num_unique));
        e = cudaGetLastError();
        // a launch that failed leaves the table in an unknown state: the
        // next call clears it again
        if (e != cudaSuccess) cudaMemsetAsync(tab + kWordReady, 0, sizeof(unsigned long long), st);
    }
    if (e != cudaSuccess) {
        char msg[200];
        std::snprintf(msg, sizeof(msg), "deduplicate_pairs_noalloc: %s", cudaGetErrorString(e));
        return pgpu::set_error_cstr(PIERCE_ERR_CUDA, msg);
    }
    return PIERCE_OK;
}
