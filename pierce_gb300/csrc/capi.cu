// C ABI of the GB300 join library (include/pierce_capi.h): contexts,
// datasets, joins, results, the launch-level seam and the dedup/scan helpers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "common.cuh"

namespace pgpu {
// join.cu
int launch_edge_rays(pierce_ctx* ctx, const DevDataset& src, const DevDataset& tgt, int mode, int precision,
                     int swap, int32_t* counts, const int64_t* offsets, uint64_t* keys, uint64_t* table,
                     uint64_t slots, const RayOpts* ro);
int launch_resolve(pierce_ctx* ctx, const DevDataset& src, const DevDataset& tgt, int swap, uint64_t* table,
                   uint64_t slots, const RayOpts* ro, uint64_t* keys_out, unsigned long long* keys_count,
                   uint64_t keys_cap);
int launch_cull(pierce_ctx* ctx, const DevDataset& src, const DevDataset& tgt, uint8_t* active, uint32_t* list,
                unsigned long long* count);
int launch_object_active(pierce_ctx* ctx, const DevDataset& src, const DevDataset& tgt, uint8_t* active);
int launch_collect_rays(pierce_ctx* ctx, const DevDataset& src, const uint8_t* active, uint32_t* list,
                        unsigned long long* count);
int launch_collect_tris(pierce_ctx* ctx, const int32_t* t2o, int64_t nt, const uint8_t* active, uint32_t* list,
                        unsigned long long* count);
int launch_chunk_cull(pierce_ctx* ctx, bool edges, const float* verts, const uint32_t* idx, const int32_t* t2o,
                      const DevDataset& src, const uint8_t* obj_active, const DevDataset& objs,
                      uint8_t* chunk_active, uint32_t* list, unsigned long long* count, float* chunk_box,
                      uint32_t* chunk_list, unsigned long long* chunk_count);
int launch_flag_list(pierce_ctx* ctx, const uint8_t* flags, int64_t n, uint32_t* list, unsigned long long* count);
int launch_soup_rays(pierce_ctx* ctx, const float4* soup, int64_t n_tris, int G, const DevDataset* filter,
                     const int32_t* obj_part, uint32_t* list, unsigned long long* count, int shard_index,
                     int shard_count, const Node4* entry_nodes4, int32_t* entries);
int launch_containment_candidates(pierce_ctx* ctx, const uint64_t* ptable, const uint32_t* parity, uint64_t pslots,
                                  uint8_t* act_a, int64_t na, uint8_t* act_b, int64_t nb);
int launch_group_incidences(pierce_ctx* ctx, const float4* soup, int64_t n_tris, int G, int step,
                            const DevDataset& tgt, unsigned long long* count);
int launch_containment_pairs(pierce_ctx* ctx, const uint64_t* ptable, const uint32_t* parity, uint64_t pslots,
                             const DevDataset& a, const DevDataset& b, uint64_t* out, unsigned long long* count,
                             uint64_t cap, unsigned long long* fallback);
int launch_object_pseudo_tris(pierce_ctx* ctx, int32_t n, uint32_t* idx, int32_t* t2o);
int launch_parity(pierce_ctx* ctx, const DevDataset& src, const DevDataset& tgt, int swap, uint64_t* table,
                  uint32_t* parity, uint64_t slots, int64_t src_lo = 0, int64_t src_hi = -1);
int launch_parity_objects(pierce_ctx* ctx, const DevDataset& src, const DevDataset& objs, const DevDataset& tgt,
                          const ColumnGrid* grid, int swap, uint64_t* table, uint32_t* parity, uint64_t slots,
                          int64_t src_lo = 0, int64_t src_hi = -1);
int launch_parity_tracking(pierce_ctx* ctx, const DevDataset& src, const DevDataset& tgt, const ColumnGrid& grid,
                           int32_t k, int32_t* ids, uint32_t* hits, uint32_t* crossed, uint32_t* overflow);
size_t column_grid_bytes(int32_t n);
int column_grid_count(pierce_ctx* ctx, const DevDataset& tgt, void* mem, const int32_t** d_total);
int column_grid_fill(pierce_ctx* ctx, const DevDataset& tgt, void* mem, int32_t* entries, ColumnGrid* g);
int compact_table(pierce_ctx* ctx, const uint64_t* table, uint64_t slots, uint64_t* out, uint64_t cap,
                  unsigned long long* d_count);
int keys_to_pairs(pierce_ctx* ctx, uint64_t* keys, int64_t n);
int pairs_to_keys(pierce_ctx* ctx, const uint64_t* pairs, uint64_t* keys, int64_t n);
int parity_emit(pierce_ctx* ctx, const uint64_t* ptable, const uint32_t* parity, uint64_t pslots, int mode,
                const uint64_t* lookup_table, uint64_t lookup_slots, const uint64_t* lookup_sorted, int64_t lookup_n,
                uint64_t* out_table, uint64_t out_slots, uint64_t* out_keys, unsigned long long* out_count,
                uint64_t out_cap);
uint64_t table_slots_for(uint64_t expected, double load_factor);
int estimate_cells(pierce_ctx* ctx, const void* a, const void* b, int n, float cell_volume, float eps, float gamma,
                   double* total);
}  // namespace pgpu

using namespace pgpu;

namespace {
// Last error message of the calling host thread.  A fixed buffer, so that
// reporting an error never allocates.
thread_local char g_err[512];

// scratch slot assignment
enum : int {
    SLOT_CUB = 0,
    SLOT_BUILD_A = 1,
    SLOT_BUILD_B = 2,
    SLOT_BUILD_C = 3,
    SLOT_BUILD_D = 4,
    SLOT_TABLE = 5,
    SLOT_KEYS = 6,
    SLOT_AUX = 7,
    SLOT_LIST_AB = 8,    // culled ray list A->B
    SLOT_LIST_BA = 9,    // culled ray list B->A
    SLOT_CULL = 10,      // active flags + counters
    SLOT_AMB = 11,       // deferred exact tests
    SLOT_EXTRA = 12,     // exactly resolved keys (two-pass)
    SLOT_RED_SOUP_A = 13,  // per-join BVH over active triangles of A
    SLOT_RED_NODES_A = 14,
    SLOT_RED_SOUP_B = 15,
    SLOT_RED_NODES_B = 16,
    SLOT_OBJ_A = 17,     // object pseudo-triangles of A (indices, ids) + their BVH
    SLOT_OBJ_B = 18,
    SLOT_TRIS_A = 19,    // active triangle lists
    SLOT_TRIS_B = 20,
    // 21, 22: learned sizing
    SLOT_CHUNK_LIST = 24,  // active chunk ids of one culling pass
    SLOT_GROUPS = 25,    // group boxes and group hierarchy soup of a grouped build
    SLOT_GRID_A = 26,    // column grids (parity candidates): A's, then B's
    SLOT_GRID_A_ENTRIES = 27,
    SLOT_GRID_B = 28,
    SLOT_GRID_B_ENTRIES = 29,
    SLOT_NODES4_A = 30,  // four-wide copies of the per-join hierarchies
    SLOT_NODES4_B = 31,
    SLOT_NODES4_OBJ_A = 32,  // ... of the object hierarchies (culling)
    SLOT_NODES4_OBJ_B = 33,
    SLOT_CONT_PARITY = 35,    // containment: parity table of B's first vertices in A
    SLOT_ENTRY_AB = 38,       // rays from triangles: entry nodes of the listed groups, A->B
    SLOT_ENTRY_BA = 39,
};
}  // namespace

namespace pgpu {

int set_error_cstr(int status, const char* msg) {
    std::snprintf(g_err, sizeof(g_err), "%s", msg ? msg : "");
    return status;
}

int set_error(int status, const std::string& msg) { return set_error_cstr(status, msg.c_str()); }

int check_cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return PIERCE_OK;
    const int st = (e == cudaErrorMemoryAllocation) ? PIERCE_ERR_OUT_OF_MEMORY : PIERCE_ERR_CUDA;
    return set_error(st, std::string(what) + ": " + cudaGetErrorString(e));
}

int device_alloc(void** p, size_t bytes, const char* what) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(PIERCE_ERR_OUT_OF_MEMORY,
                         std::string("cudaMalloc(") + std::to_string(bytes) + ") for " + what + ": " +
                             cudaGetErrorString(e));
    }
    return PIERCE_OK;
}

// Leaf size of a join's per-join hierarchies over dataset ds: the join's
// own setting, else the dataset's when above one, else 4 (groups of four
// consecutive triangles: the fastest on the measured workloads, and a
// quarter of the build memory of single-triangle leaves).
static int join_leaf(const pierce_join_opts& o, const pierce_dataset* ds) {
    if (o.leaf_size > 0) return o.leaf_size;
    return ds->leaf_size > 1 ? ds->leaf_size : 4;
}

// Free every scratch slot that the running join (generation `keep_gen`)
// has not used, and the pool's unused memory.  keep_gen 0: free all slots.
static void release_idle_memory(pierce_ctx* ctx, uint64_t keep_gen) {
    cudaDeviceSynchronize();
    for (int i = 0; i < kScratchSlots; ++i) {
        if (!ctx->scratch[i] || (keep_gen && ctx->scratch_used[i] == keep_gen)) continue;
        cudaFree(ctx->scratch[i]);
        ctx->scratch[i] = nullptr;
        ctx->scratch_bytes[i] = 0;
    }
    if (ctx->pool) cudaMemPoolTrimTo(ctx->pool, 0);
}

int dataset_array(pierce_ctx* ctx, void** p, size_t bytes, cudaStream_t stream, const char* what) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMallocFromPoolAsync(p, bytes, ctx->pool, stream);
    if (e == cudaErrorMemoryAllocation) {
        // the joins' scratch and the memory other datasets returned to the
        // pool go back to the device first (no join is running)
        cudaGetLastError();
        release_idle_memory(ctx, 0);
        e = cudaMallocFromPoolAsync(p, bytes, ctx->pool, stream);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return set_error(e == cudaErrorMemoryAllocation ? PIERCE_ERR_OUT_OF_MEMORY : PIERCE_ERR_CUDA,
                         std::string("device allocation (") + std::to_string(bytes) + ") for " + what + ": " +
                             cudaGetErrorString(e));
    }
    return PIERCE_OK;
}

// Only called with the device idle (pierce_dataset_destroy synchronises
// first), so the legacy stream orders nothing that still runs.
void dataset_free(void* p) {
    if (p) cudaFreeAsync(p, 0);
}

int host_value(pierce_ctx* ctx, const void* dptr, int bytes, int64_t* out, const char* what) {
    GraphPlan* g = ctx->plan;
    if (g && g->mode == 2) {
        if (g->cursor >= g->values.size() || g->widths[g->cursor] != bytes)
            return set_error(PIERCE_ERR_CUDA, std::string("join graph capture left its plan at ") + what);
        cudaMemcpyAsync(g->h_check + g->cursor, dptr, (size_t)bytes, cudaMemcpyDeviceToHost, ctx->stream);
        *out = g->values[g->cursor++];
        return PIERCE_OK;
    }
    int64_t* slot = ctx->h_small + 7;
    *slot = 0;
    if (int s = check_cuda(cudaMemcpyAsync(slot, dptr, (size_t)bytes, cudaMemcpyDeviceToHost, ctx->stream), what))
        return s;
    if (int s = check_cuda(cudaStreamSynchronize(ctx->stream), what)) return s;
    int64_t v = *slot;
    if (bytes == 4) {
        int32_t w;
        std::memcpy(&w, slot, 4);
        v = w;
    }
    if (g && g->mode == 1) {
        g->values.push_back(v);
        g->widths.push_back(bytes);
    }
    *out = v;
    return PIERCE_OK;
}

int result_alloc(pierce_ctx* ctx, void** p, size_t bytes) {
    GraphPlan* g = ctx->plan;
    if (g && g->mode == 2) {
        if (g->buf_cursor >= g->buffers.size() || g->buffer_bytes[g->buf_cursor] < bytes)
            return set_error(PIERCE_ERR_CUDA, "join graph capture: result buffer differs from its plan");
        *p = g->buffers[g->buf_cursor++];
        return PIERCE_OK;
    }
    if (int s = device_alloc(p, bytes, "result")) return s;
    if (g && g->mode == 1) {
        g->buffers.push_back(*p);
        g->buffer_bytes.push_back(bytes);
    }
    return PIERCE_OK;
}

int scratch(pierce_ctx* ctx, int slot, size_t bytes, void** out) {
    if (bytes == 0) bytes = 16;
    if (ctx->scratch_bytes[slot] < bytes && capturing(ctx))
        return set_error(PIERCE_ERR_CUDA, "join graph capture: scratch would grow");
    ctx->scratch_used[slot] = ctx->scratch_gen;
    if (ctx->scratch_bytes[slot] < bytes) {
        if (ctx->scratch[slot]) {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(ctx->scratch[slot]);
            ctx->scratch[slot] = nullptr;
            ctx->scratch_bytes[slot] = 0;
        }
        size_t want = bytes + bytes / 8;  // headroom against repeated growth
        if (device_alloc(&ctx->scratch[slot], want, "scratch") != PIERCE_OK) {
            // slots earlier joins left behind and the pool's unused memory go
            // back to the device first (not while a join graph is planned:
            // the plan holds on to its buffers)
            if (ctx->plan) return PIERCE_ERR_OUT_OF_MEMORY;
            release_idle_memory(ctx, ctx->scratch_gen ? ctx->scratch_gen : ~0ull);
            if (int s = device_alloc(&ctx->scratch[slot], want, "scratch")) return s;
        }
        if (!ctx->scratch[slot]) return PIERCE_ERR_OUT_OF_MEMORY;
        ctx->scratch_bytes[slot] = want;
    }
    *out = ctx->scratch[slot];
    return PIERCE_OK;
}

}  // namespace pgpu

// ---------------------------------------------------------------- kernels --

// Edge upload: a warp per 32-edge chunk packs its edges (start + source
// object bits, end), copies the source ids, writes the chunk's box (the
// values k_chunk_boxes computes) and clears *grouped when a source id
// decreases.  The inputs may be pinned host memory the device reads in
// place, so the transfer and the packing are one pass.
__global__ void __launch_bounds__(256) k_upload_edges(const float* s, const float* e, const int32_t* src, int64_t n,
                                                      float4* __restrict__ out, int32_t* __restrict__ src_out,
                                                      float* __restrict__ chunk_box, int32_t* __restrict__ grouped) {
    const int lane = threadIdx.x & 31;
    const int64_t chunks = (n + 31) / 32;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t c = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); c < chunks; c += warps) {
        const int64_t i = c * 32 + lane;
        float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
        int32_t o = 0;
        if (i < n) {
            const float sx = s[3 * i], sy = s[3 * i + 1], sz = s[3 * i + 2];
            const float ex = e[3 * i], ey = e[3 * i + 1], ez = e[3 * i + 2];
            o = src[i];
            out[2 * i] = make_float4(sx, sy, sz, __int_as_float(o));
            out[2 * i + 1] = make_float4(ex, ey, ez, 0.0f);
            src_out[i] = o;
            lo[0] = fminf(sx, ex); lo[1] = fminf(sy, ey); lo[2] = fminf(sz, ez);
            hi[0] = fmaxf(sx, ex); hi[1] = fmaxf(sy, ey); hi[2] = fmaxf(sz, ez);
        }
        int32_t next = __shfl_down_sync(0xFFFFFFFFu, o, 1);
        if (lane == 31 && i + 1 < n) next = src[i + 1];
        if (i + 1 < n && next < o) atomicAnd(grouped, 0);
        for (int k = 0; k < 3; ++k)
            for (int off = 16; off > 0; off >>= 1) {
                lo[k] = fminf(lo[k], __shfl_xor_sync(0xFFFFFFFFu, lo[k], off));
                hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xFFFFFFFFu, hi[k], off));
            }
        if (lane < 6) chunk_box[6 * c + lane] = lane < 3 ? lo[lane] : hi[lane - 3];
    }
}

// A pointer the device can read for array `h`: the device alias of pinned
// (registered) host memory, or device memory itself; nullptr for pageable
// host memory, which goes through the copy engines (they read it at the
// link's full rate).
static const void* device_readable(const void* h) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return h;
    if (a.type == cudaMemoryTypeHost) return a.devicePointer;
    return nullptr;
}

__global__ void k_pack_edges(const float* __restrict__ s, const float* __restrict__ e, const int32_t* __restrict__ src,
                             int64_t n, float4* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        out[2 * i] = make_float4(s[3 * i], s[3 * i + 1], s[3 * i + 2], __int_as_float(src[i]));
        out[2 * i + 1] = make_float4(e[3 * i], e[3 * i + 1], e[3 * i + 2], 0.0f);
    }
}

// Per-triangle object ids from object ranges: triangle t belongs to the
// object o with off[o] <= t < off[o + 1] (binary search; empty objects skipped).
__global__ void k_fill_t2o(const int64_t* __restrict__ off, int32_t nobj, int64_t nt, int32_t* __restrict__ t2o) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
        int32_t lo = 0, hi = nobj;  // off[lo] <= t < off[hi]
        while (hi - lo > 1) {
            const int32_t mid = (lo + hi) >> 1;
            if (__ldg(off + mid) <= t) lo = mid;
            else hi = mid;
        }
        t2o[t] = lo;
    }
}

__global__ void k_max_i32(const int32_t* __restrict__ v, int64_t n, int32_t* out) {
    int32_t m = -1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = max(m, v[i]);
    for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_xor_sync(0xFFFFFFFFu, m, off));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// ------------------------------------------------------------ host helpers --

static int grid_for(pierce_ctx* ctx, int64_t n, int block) {
    int64_t b = (n + block - 1) / block;
    const int64_t cap = (int64_t)ctx->sm_count * 16;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

static int sync_ctx(pierce_ctx* ctx, const char* what) {
    if (capturing(ctx)) return PIERCE_OK;  // a captured join synchronises after its replay
    return check_cuda(cudaStreamSynchronize(ctx->stream), what);
}

// Translate device error bits into a status (the bits are cleared).  Inside
// a captured join the bits of the planning run stand in, and the replay
// compares the device's bits with them.
static int read_device_error(pierce_ctx* ctx, uint32_t* bits_out) {
    int64_t v = 0;
    if (int s = host_value(ctx, ctx->d_err, 4, &v, "device error word")) return s;
    *bits_out = (uint32_t)v;
    cudaMemsetAsync(ctx->d_err, 0, sizeof(uint32_t), ctx->stream);
    return PIERCE_OK;
}

struct EventTimer {
    std::vector<cudaEvent_t> ev;
    std::vector<std::pair<int, int>> spans;  // (begin idx, end idx) per label
    std::vector<double*> targets;
    cudaStream_t st;
    bool off = false;  // no events inside a captured join
    explicit EventTimer(cudaStream_t s) : st(s) {}
    int record() {
        if (off) return -1;
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, st);
        ev.push_back(e);
        return (int)ev.size() - 1;
    }
    void span(int b, int e, double* target) {
        if (off || b < 0 || e < 0) return;
        spans.emplace_back(b, e);
        targets.push_back(target);
    }
    void resolve() {
        for (size_t i = 0; i < spans.size(); ++i) {
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, ev[spans[i].first], ev[spans[i].second]);
            *targets[i] += ms;
        }
    }
    ~EventTimer() {
        for (auto e : ev) cudaEventDestroy(e);
    }
};

// ------------------------------------------------- dataset construction --

namespace pgpu {

int dataset_alloc(pierce_dataset* ds, cudaStream_t stream) {
    const int32_t nobj = ds->num_objects;
    const size_t vb = 12 * ds->nv, ib = 12 * ds->nt, ob = 4 * ds->nt;
    pierce_ctx* c = ds->ctx;
    if (int s = dataset_array(c, (void**)&ds->d_vertices, vb, stream, "vertices")) return s;
    if (int s = dataset_array(c, (void**)&ds->d_indices, ib, stream, "indices")) return s;
    if (int s = dataset_array(c, (void**)&ds->d_tri_to_object, ob, stream, "triangle to object")) return s;
    if (int s = dataset_array(c, (void**)&ds->d_edges, 32 * ds->ne, stream, "edges")) return s;
    if (int s = dataset_array(c, (void**)&ds->d_edge_src, 4 * std::max<uint64_t>(ds->ne, 1), stream, "edge sources"))
        return s;
    if (int s = dataset_array(c, (void**)&ds->d_first_vertex, 16 * (size_t)std::max(nobj, 1), stream,
                              "first vertices"))
        return s;
    if (int s = dataset_array(c, (void**)&ds->d_obj_box, 24 * (size_t)std::max(nobj, 1), stream, "object boxes"))
        return s;
    if (int s = dataset_array(c, (void**)&ds->d_obj_range, 8 * (size_t)std::max(nobj, 1), stream, "object ranges"))
        return s;
    const size_t tcb = 24 * ((ds->nt + 31) / 32 + 1), ecb = 24 * ((ds->ne + 31) / 32 + 1);
    if (int s = dataset_array(c, (void**)&ds->d_tri_chunk_box, tcb, stream, "triangle chunk boxes")) return s;
    if (int s = dataset_array(c, (void**)&ds->d_edge_chunk_box, ecb, stream, "edge chunk boxes")) return s;
    ds->device_bytes = vb + ib + ob + 36 * ds->ne + 48 * (size_t)nobj + tcb + ecb;
    return PIERCE_OK;
}

int dataset_finish(pierce_ctx* ctx, pierce_dataset* ds, const pierce_tuning* tuning, cudaEvent_t edges_ready,
                   const int32_t* grouped_flag) {
    if (int s = prepare_objects(ctx, ds, edges_ready, grouped_flag)) return s;
    pierce_tuning t;
    pierce_default_tuning(&t);
    if (tuning) t = *tuning;
    // a leaf size above one also applies to the per-join hierarchies
    ds->leaf_size = std::min(std::max(t.leaf_size, 1), 16);
    if (t.defer_build) return sync_ctx(ctx, "dataset upload");
    return build_bvh(ctx, ds, t.leaf_size);
}

}  // namespace pgpu

// ------------------------------------------------------------------ C ABI --

extern "C" {

const char* pierce_last_error(void) { return g_err; }

const char* pierce_status_string(int status) {
    switch (status) {
        case PIERCE_OK: return "ok";
        case PIERCE_ERR_INVALID_ARGUMENT: return "invalid argument";
        case PIERCE_ERR_CUDA: return "CUDA error";
        case PIERCE_ERR_OUT_OF_MEMORY: return "out of device memory";
        case PIERCE_ERR_NO_DEVICE: return "no CUDA device";
        case PIERCE_ERR_HASH_FULL: return "hash table full";
        case PIERCE_ERR_STACK_OVERFLOW: return "traversal stack overflow";
        case PIERCE_ERR_OUTPUT_OVERFLOW: return "output buffer overflow";
        case PIERCE_ERR_QUEUE_TIMEOUT: return "work queue wait timed out";
        case PIERCE_ERR_NOT_BUILT: return "dataset not built";
        default: return "unknown status";
    }
}

void pierce_default_tuning(pierce_tuning* t) {
    if (!t) return;
    t->leaf_size = 1;
    t->block_size = 128;
    t->sort_rays = 0;
    t->cull_objects = 0;
    t->defer_build = 0;
    t->skip_edges = 0;
}

void pierce_default_join_opts(pierce_join_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->predicate = PIERCE_OVERLAP;
    o->direction = PIERCE_BOTH;
    o->sizing = PIERCE_SIZING_HASH;
    o->precision = PIERCE_EXACT;
    o->expected_pairs = 0;
    o->hash_table_slots = 0;
    o->hash_load_factor = 0.5;
    o->output_safety = 1.2;
    o->include_overlap_pairs = 0;
    o->max_retries = 4;
    o->cull_objects = 1;
    o->defer_exact = 1;
    o->active_bvh = 1;
}

int pierce_ctx_create(int device, pierce_ctx** out) {
    if (!out) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "ctx_create: null out");
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return set_error(PIERCE_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= n) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "ctx_create: bad device index");
    if (int s = check_cuda(cudaSetDevice(device), "cudaSetDevice")) return s;
    pierce_ctx* ctx = new pierce_ctx();
    ctx->device = device;
    int st = check_cuda(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "stream create");
    if (!st) st = device_alloc((void**)&ctx->d_err, sizeof(uint32_t), "error word");
    if (!st) st = device_alloc((void**)&ctx->d_counters, sizeof(DevCounters), "counters");
    if (!st) st = check_cuda(cudaMallocHost((void**)&ctx->h_err, sizeof(uint32_t)), "pinned");
    if (!st) st = check_cuda(cudaMallocHost((void**)&ctx->h_counters, sizeof(DevCounters)), "pinned");
    if (!st) st = check_cuda(cudaMallocHost((void**)&ctx->h_small, 8 * sizeof(int64_t)), "pinned");
    if (!st) st = check_cuda(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device), "attr");
    if (!st) st = check_cuda(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking), "stream create");
    if (!st) st = check_cuda(cudaEventCreateWithFlags(&ctx->ev_tris, cudaEventDisableTiming), "event create");
    if (!st) st = check_cuda(cudaEventCreateWithFlags(&ctx->ev_edges, cudaEventDisableTiming), "event create");
    if (!st) st = device_alloc((void**)&ctx->d_upload_flag, 16, "upload flag");
    if (!st) {
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        st = check_cuda(cudaMemPoolCreate(&ctx->pool, &props), "memory pool");
        if (!st) {
            // keep up to a quarter of the device's memory of freed arrays for
            // the next datasets; beyond that the pool returns memory at
            // synchronisation points (and an allocation short of memory trims
            // it first)
            size_t free_b = 0, total_b = 0;
            if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
                cudaGetLastError();
                total_b = (size_t)64 << 30;
            }
            uint64_t keep = (uint64_t)total_b / 4;
            st = check_cuda(cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep), "pool");
        }
    }
    if (!st) st = check_cuda(cudaMemsetAsync(ctx->d_err, 0, sizeof(uint32_t), ctx->stream), "memset");
    if (!st) st = sync_ctx(ctx, "ctx init");
    if (st) {
        pierce_ctx_destroy(ctx);
        return st;
    }
    *out = ctx;
    return PIERCE_OK;
}

void pierce_ctx_destroy(pierce_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    for (int i = 0; i < kScratchSlots; ++i)
        if (ctx->scratch[i]) cudaFree(ctx->scratch[i]);
    if (ctx->d_upload_flag) cudaFree(ctx->d_upload_flag);
    if (ctx->ev_tris) cudaEventDestroy(ctx->ev_tris);
    if (ctx->ev_edges) cudaEventDestroy(ctx->ev_edges);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    // arrays of datasets that outlive the context stay valid; the pool's
    // memory is released once they are freed
    if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
    if (ctx->d_err) cudaFree(ctx->d_err);
    if (ctx->d_counters) cudaFree(ctx->d_counters);
    if (ctx->h_err) cudaFreeHost(ctx->h_err);
    if (ctx->h_counters) cudaFreeHost(ctx->h_counters);
    if (ctx->h_small) cudaFreeHost(ctx->h_small);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int pierce_ctx_synchronize(pierce_ctx* ctx) {
    if (!ctx) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "null ctx");
    return sync_ctx(ctx, "synchronize");
}

void* pierce_ctx_stream(pierce_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

uint64_t pierce_ctx_kernel_launches(const pierce_ctx* ctx) { return ctx ? ctx->launches : 0; }

int pierce_ctx_release_scratch(pierce_ctx* ctx) {
    if (!ctx) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "ctx_release_scratch: null argument");
    cudaSetDevice(ctx->device);
    if (int s = check_cuda(cudaStreamSynchronize(ctx->stream), "release scratch")) return s;
    for (int i = 0; i < kScratchSlots; ++i) {
        if (ctx->scratch[i]) cudaFree(ctx->scratch[i]);
        ctx->scratch[i] = nullptr;
        ctx->scratch_bytes[i] = 0;
    }
    // and the arrays of destroyed datasets that the pool still holds
    if (ctx->pool) cudaMemPoolTrimTo(ctx->pool, 0);
    return PIERCE_OK;
}

int pierce_device_memory(pierce_ctx* ctx, uint64_t* free_bytes, uint64_t* total_bytes) {
    if (!ctx || !free_bytes || !total_bytes) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "device_memory: null");
    cudaSetDevice(ctx->device);
    size_t f = 0, t = 0;
    if (int s = check_cuda(cudaMemGetInfo(&f, &t), "cudaMemGetInfo")) return s;
    *free_bytes = f;
    *total_bytes = t;
    return PIERCE_OK;
}

// ---- datasets ---------------------------------------------------------------

void pierce_dataset_destroy(pierce_dataset* ds) {
    if (!ds) return;
    // The device id is a copy, so a dataset outliving its context is still
    // released; the device-wide synchronisation covers work still queued.
    cudaSetDevice(ds->device);
    cudaDeviceSynchronize();
    void* ptrs[] = {ds->d_vertices, ds->d_indices,  ds->d_tri_to_object, ds->d_edges,  ds->d_edge_src,
                    ds->d_soup,     ds->d_nodes,    ds->d_first_vertex,  ds->d_obj_box, ds->d_obj_part,
                    ds->d_part_roots, ds->d_obj_range, ds->d_tri_chunk_box, ds->d_edge_chunk_box,
                    ds->d_obj_hier, ds->d_grid, ds->d_grid_entries};
    for (void* p : ptrs) dataset_free(p);
    // the frees complete now, so the next dataset of the context reuses the memory
    cudaStreamSynchronize(0);
    delete ds;
}

int pierce_dataset_set_partitions(pierce_ctx* ctx, pierce_dataset* ds, const int32_t* obj_part, int32_t num_parts) {
    if (!ctx || !ds || num_parts < 0 || (num_parts > 0 && ds->num_objects > 0 && !obj_part))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "dataset_set_partitions: invalid argument");
    if (num_parts >= (1 << 30))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "dataset_set_partitions: at most 2^30 - 1 partitions");
    for (int32_t o = 0; num_parts > 0 && o < ds->num_objects; ++o)
        if (obj_part[o] < 0 || obj_part[o] >= num_parts)
            return set_error(PIERCE_ERR_INVALID_ARGUMENT, "dataset_set_partitions: partition id out of range");
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaDeviceSynchronize();  // dataset_free needs an idle device
    dataset_free(ds->d_obj_part);
    dataset_free(ds->d_part_roots);
    dataset_free(ds->d_obj_hier);  // the object hierarchy follows the partitions
    dataset_free(ds->d_grid);
    dataset_free(ds->d_grid_entries);
    ds->d_obj_part = nullptr;
    ds->d_part_roots = nullptr;
    ds->d_obj_hier = nullptr;
    ds->obj_hier_ready = 0;
    ds->d_grid = nullptr;
    ds->d_grid_entries = nullptr;
    ds->grid_ready = 0;
    ds->num_parts = 0;
    const bool was_built = ds->built != 0;
    ds->built = 0;
    if (num_parts > 0) {
        const size_t nobj = (size_t)std::max(ds->num_objects, 1);
        if (int s = dataset_array(ctx, (void**)&ds->d_obj_part, 4 * nobj, ctx->stream, "object partitions")) return s;
        if (int s = dataset_array(ctx, (void**)&ds->d_part_roots, 8 * (size_t)num_parts, ctx->stream,
                                  "partition roots"))
            return s;
        if (ds->num_objects > 0)
            if (int s = check_cuda(cudaMemcpyAsync(ds->d_obj_part, obj_part, 4 * (size_t)ds->num_objects,
                                                   cudaMemcpyHostToDevice, ctx->stream),
                                   "copy partitions"))
                return s;
        ds->num_parts = num_parts;
    }
    if (was_built) return build_bvh(ctx, ds, ds->leaf_size);
    return sync_ctx(ctx, "set partitions");
}

int pierce_dataset_build(pierce_ctx* ctx, pierce_dataset* ds, const pierce_tuning* tuning) {
    if (!ctx || !ds) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "dataset_build: null argument");
    pierce_tuning t;
    pierce_default_tuning(&t);
    if (tuning) t = *tuning;
    return build_bvh(ctx, ds, t.leaf_size);
}

// The per-triangle object ids of a new dataset on `stream`: copied from the
// view, or written from its object ranges (the offsets go over in one copy).
static int upload_object_ids(pierce_ctx* ctx, pierce_dataset* ds, const pierce_mesh_view* v, cudaMemcpyKind kind,
                             cudaStream_t stream) {
    if (!v->object_offsets)
        return check_cuda(cudaMemcpyAsync(ds->d_tri_to_object, v->tri_to_object, 4 * ds->nt, kind, stream), "copy t2o");
    const size_t bytes = 8 * ((size_t)ds->num_objects + 1);
    void* d_off = nullptr;
    if (int s = check_cuda(cudaMallocFromPoolAsync(&d_off, bytes, ctx->pool, stream), "object offsets")) return s;
    if (int s = check_cuda(cudaMemcpyAsync(d_off, v->object_offsets, bytes, cudaMemcpyHostToDevice, stream),
                           "copy object offsets"))
        return s;
    k_fill_t2o<<<grid_for(ctx, (int64_t)ds->nt, 256), 256, 0, stream>>>((const int64_t*)d_off, ds->num_objects,
                                                                        (int64_t)ds->nt, ds->d_tri_to_object);
    ctx->launches += 1;
    if (int s = check_cuda(cudaGetLastError(), "object ids from ranges")) return s;
    return check_cuda(cudaFreeAsync(d_off, stream), "object offsets");
}

int pierce_dataset_create(pierce_ctx* ctx, const pierce_mesh_view* v, int memory, const pierce_tuning* tuning,
                          pierce_dataset** out) {
    if (!ctx || !v || !out) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "dataset_create: null argument");
    *out = nullptr;
    // skip_edges: the edge arrays are neither read nor uploaded (the joins
    // take their rays from the triangles)
    const bool skip_edges = tuning && tuning->skip_edges;
    const uint64_t num_edges = skip_edges ? 0 : v->num_edges;
    const bool ranges = v->object_offsets != nullptr;
    if ((v->num_vertices && !v->vertices) || (v->num_triangles && (!v->indices || (!v->tri_to_object && !ranges))) ||
        (num_edges && (!v->edge_starts || !v->edge_ends || !v->edge_src)))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "dataset_create: missing array");
    if (ranges) {
        // object ranges: a count is given, the offsets run from 0 to the
        // triangle count without decreasing
        if (v->num_objects < 0)
            return set_error(PIERCE_ERR_INVALID_ARGUMENT, "dataset_create: object ranges need num_objects");
        const int64_t* off = v->object_offsets;
        bool ok = off[0] == 0 && off[v->num_objects] == (int64_t)v->num_triangles;
        for (int32_t o = 0; ok && o < v->num_objects; ++o) ok = off[o] <= off[o + 1];
        if (!ok)
            return set_error(PIERCE_ERR_INVALID_ARGUMENT,
                             "dataset_create: object offsets must rise from 0 to the triangle count");
    }
    if (v->num_triangles >= (1ull << 31) || num_edges >= (1ull << 40) || v->num_vertices >= (1ull << 32))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "dataset_create: dataset too large for 32-bit ids");
    cudaSetDevice(ctx->device);
    const cudaMemcpyKind kind = memory == PIERCE_DEVICE_MEMORY ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    pierce_dataset* ds = new pierce_dataset();
    ds->ctx = ctx;
    ds->device = ctx->device;
    ds->nv = v->num_vertices;
    ds->nt = v->num_triangles;
    ds->ne = num_edges;
    cudaStream_t st = ctx->stream;
    int s = PIERCE_OK;
    do {
        // object count
        int32_t nobj = v->num_objects;
        if (nobj < 0) {
            if (memory == PIERCE_HOST_MEMORY) {
                nobj = 0;
                for (uint64_t i = 0; i < ds->nt; ++i) nobj = std::max(nobj, v->tri_to_object[i] + 1);
            } else if (ds->nt > 0) {
                void* p = nullptr;
                if ((s = scratch(ctx, SLOT_AUX, sizeof(int32_t), &p))) break;
                cudaMemsetAsync(p, 0xFF, sizeof(int32_t), st);
                k_max_i32<<<grid_for(ctx, (int64_t)ds->nt, 256), 256, 0, st>>>(v->tri_to_object, (int64_t)ds->nt,
                                                                                 (int32_t*)p);
                ctx->launches += 1;
                cudaMemcpyAsync(ctx->h_small, p, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
                if ((s = sync_ctx(ctx, "object count"))) break;
                nobj = *reinterpret_cast<int32_t*>(ctx->h_small) + 1;
            } else {
                nobj = 0;
            }
        }
        ds->num_objects = nobj;
        // Pipelined upload when the device reads the edge arrays in place
        // (pinned host memory or device memory):
        // the triangle-side copies, then the edge upload kernel, run on the
        // copy stream; the object preparation of the triangles starts on the
        // context stream as soon as they have arrived (ev_tris) and overlaps
        // the edge transfer.  Otherwise everything runs on the context stream
        // through staging buffers.
        const void* es = nullptr;
        const void* ee = nullptr;
        const void* esrc = nullptr;
        if (ds->ne) {
            es = device_readable(v->edge_starts);
            ee = device_readable(v->edge_ends);
            esrc = device_readable(v->edge_src);
        }
        const bool direct = ds->ne == 0 || (es && ee && esrc);
        if (direct) {
            cudaStream_t cs = ctx->copy_stream;
            if ((s = dataset_alloc(ds, cs))) break;
            const size_t vb = 12 * ds->nv, ib = 12 * ds->nt, ob = 4 * ds->nt;
            if (vb && (s = check_cuda(cudaMemcpyAsync(ds->d_vertices, v->vertices, vb, kind, cs), "copy vertices")))
                break;
            if (ib && (s = check_cuda(cudaMemcpyAsync(ds->d_indices, v->indices, ib, kind, cs), "copy indices")))
                break;
            if (ob && (s = upload_object_ids(ctx, ds, v, kind, cs))) break;
            if ((s = check_cuda(cudaEventRecord(ctx->ev_tris, cs), "upload event"))) break;
            if ((s = check_cuda(cudaMemsetAsync(ctx->d_upload_flag, 1, sizeof(int32_t), cs), "upload flag"))) break;
            if (ds->ne) {
                const int64_t chunks = (int64_t)((ds->ne + 31) / 32);
                const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((chunks + 7) / 8, ctx->sm_count * 4));
                k_upload_edges<<<blocks, 256, 0, cs>>>((const float*)es, (const float*)ee, (const int32_t*)esrc,
                                                       (int64_t)ds->ne, ds->d_edges, ds->d_edge_src,
                                                       ds->d_edge_chunk_box, ctx->d_upload_flag);
                ctx->launches += 1;
                if ((s = check_cuda(cudaGetLastError(), "upload edges"))) break;
            }
            if ((s = check_cuda(cudaEventRecord(ctx->ev_edges, cs), "upload event"))) break;
            if ((s = check_cuda(cudaStreamWaitEvent(st, ctx->ev_tris, 0), "upload wait"))) break;
            s = dataset_finish(ctx, ds, tuning, ctx->ev_edges, ctx->d_upload_flag);
            // the caller's arrays are free to change once this returns
            if (int s2 = check_cuda(cudaStreamSynchronize(cs), "dataset upload")) s = s ? s : s2;
            break;
        }
        if ((s = dataset_alloc(ds, st))) break;
        const size_t vb = 12 * ds->nv, ib = 12 * ds->nt, ob = 4 * ds->nt;
        if (vb && (s = check_cuda(cudaMemcpyAsync(ds->d_vertices, v->vertices, vb, kind, st), "copy vertices"))) break;
        if (ib && (s = check_cuda(cudaMemcpyAsync(ds->d_indices, v->indices, ib, kind, st), "copy indices"))) break;
        if (ob && (s = upload_object_ids(ctx, ds, v, kind, st))) break;
        if (ds->ne) {
            void *ps = nullptr, *pe = nullptr;
            void* po = ds->d_edge_src;
            if ((s = scratch(ctx, SLOT_BUILD_A, 12 * ds->ne, &ps))) break;
            if ((s = scratch(ctx, SLOT_BUILD_B, 12 * ds->ne, &pe))) break;
            if ((s = check_cuda(cudaMemcpyAsync(ps, v->edge_starts, 12 * ds->ne, kind, st), "copy edge starts"))) break;
            if ((s = check_cuda(cudaMemcpyAsync(pe, v->edge_ends, 12 * ds->ne, kind, st), "copy edge ends"))) break;
            if ((s = check_cuda(cudaMemcpyAsync(po, v->edge_src, 4 * ds->ne, kind, st), "copy edge src"))) break;
            k_pack_edges<<<grid_for(ctx, (int64_t)ds->ne, 256), 256, 0, st>>>((const float*)ps, (const float*)pe,
                                                                               (const int32_t*)po, (int64_t)ds->ne,
                                                                               ds->d_edges);
            ctx->launches += 1;
            if ((s = check_cuda(cudaGetLastError(), "pack edges"))) break;
        }
        if ((s = dataset_finish(ctx, ds, tuning))) break;
    } while (0);
    if (s) {
        pierce_dataset_destroy(ds);
        return s;
    }
    *out = ds;
    return PIERCE_OK;
}

int pierce_dataset_download(pierce_ctx* ctx, const pierce_dataset* ds, float* vertices, uint32_t* indices,
                            int32_t* tri_to_object, float* edge_starts, float* edge_ends, int32_t* edge_src) {
    if (!ctx || !ds) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "dataset_download: null argument");
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    const cudaMemcpyKind d2h = cudaMemcpyDeviceToHost;
    if (vertices && ds->nv)
        if (int s = check_cuda(cudaMemcpyAsync(vertices, ds->d_vertices, 12 * ds->nv, d2h, st), "download vertices"))
            return s;
    if (indices && ds->nt)
        if (int s = check_cuda(cudaMemcpyAsync(indices, ds->d_indices, 12 * ds->nt, d2h, st), "download indices"))
            return s;
    if (tri_to_object && ds->nt)
        if (int s = check_cuda(cudaMemcpyAsync(tri_to_object, ds->d_tri_to_object, 4 * ds->nt, d2h, st),
                               "download t2o"))
            return s;
    if (edge_src && ds->ne)
        if (int s = check_cuda(cudaMemcpyAsync(edge_src, ds->d_edge_src, 4 * ds->ne, d2h, st), "download edge src"))
            return s;
    std::vector<float4> packed;
    if ((edge_starts || edge_ends) && ds->ne) {
        packed.resize(2 * ds->ne);
        if (int s = check_cuda(cudaMemcpyAsync(packed.data(), ds->d_edges, 32 * ds->ne, d2h, st), "download edges"))
            return s;
    }
    if (int s = sync_ctx(ctx, "dataset download")) return s;
    for (uint64_t i = 0; i < (packed.empty() ? 0 : ds->ne); ++i) {
        const float4 a = packed[2 * i], b = packed[2 * i + 1];
        if (edge_starts) {
            edge_starts[3 * i] = a.x;
            edge_starts[3 * i + 1] = a.y;
            edge_starts[3 * i + 2] = a.z;
        }
        if (edge_ends) {
            edge_ends[3 * i] = b.x;
            edge_ends[3 * i + 1] = b.y;
            edge_ends[3 * i + 2] = b.z;
        }
    }
    return PIERCE_OK;
}

int pierce_dataset_info_get(const pierce_dataset* ds, pierce_dataset_info* out) {
    if (!ds || !out) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "dataset_info: null argument");
    std::memset(out, 0, sizeof(*out));
    out->num_vertices = ds->nv;
    out->num_triangles = ds->nt;
    out->num_edges = ds->ne;
    out->num_objects = ds->num_objects;
    out->num_parts = ds->num_parts;
    out->objects_contiguous = ds->contiguous;
    out->built = ds->built;
    out->num_nodes = ds->num_nodes;
    out->device_bytes = ds->device_bytes;
    out->ms_build = ds->ms_build;
    for (int k = 0; k < 3; ++k) {
        out->bounds_lo[k] = ds->lo[k];
        out->bounds_hi[k] = ds->hi[k];
    }
    return PIERCE_OK;
}

// ---- results ----------------------------------------------------------------

int pierce_result_count(const pierce_result* r, uint64_t* count) {
    if (!r || !count) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "result_count: null argument");
    *count = r->count;
    return PIERCE_OK;
}

int pierce_result_containment_count(const pierce_result* r, uint64_t* count) {
    if (!r || !count) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "result_containment_count: null argument");
    *count = r->containment_count;
    return PIERCE_OK;
}

const pierce_pair* pierce_result_device_pairs(const pierce_result* r) { return r ? r->d_pairs : nullptr; }

int pierce_result_copy(pierce_ctx* ctx, const pierce_result* r, pierce_pair* host_out, uint64_t capacity) {
    if (!ctx || !r || (!host_out && capacity)) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "result_copy: null");
    const uint64_t n = std::min(capacity, r->count);
    if (n == 0) return PIERCE_OK;
    if (int s = check_cuda(cudaMemcpyAsync(host_out, r->d_pairs, n * sizeof(pierce_pair), cudaMemcpyDeviceToHost,
                                           ctx->stream),
                           "result copy"))
        return s;
    if (int s = sync_ctx(ctx, "result copy")) return s;
    return r->count > capacity ? set_error(PIERCE_ERR_OUTPUT_OVERFLOW, "result_copy: capacity below pair count")
                               : PIERCE_OK;
}

void pierce_result_destroy(pierce_result* r) {
    if (!r) return;
    if (r->d_pairs) cudaFree(r->d_pairs);
    delete r;
}

}  // extern "C"

// ---- join orchestration ------------------------------------------------------

namespace {

// Round a scratch cursor up to a 256-byte boundary.
static inline void soup_align(char*& q) { q += (256 - ((uintptr_t)q & 255)) & 255; }

struct Join {
    pierce_ctx* ctx;
    pierce_dataset* A;
    pierce_dataset* B;
    pierce_join_opts o;
    pierce_stats st;
    EventTimer timer;
    bool ab, ba;
    Join(pierce_ctx* c, pierce_dataset* a, pierce_dataset* b, const pierce_join_opts& opts)
        : ctx(c), A(a), B(b), o(opts), timer(c->stream) {
        ++c->scratch_gen;
        std::memset(&st, 0, sizeof(st));
        timer.off = capturing(c);
        ab = o.direction == PIERCE_BOTH || o.direction == PIERCE_MESH1_TO_MESH2;
        ba = o.direction == PIERCE_BOTH || o.direction == PIERCE_MESH2_TO_MESH1;
    }

    // Per-join state of the tuned edge-ray path: culled ray lists per
    // direction and the queue of deferred exact tests.
    bool listed[2] = {false, false};
    uint32_t* list[2] = {nullptr, nullptr};
    // rays from triangles, per direction: the source side's per-join soup
    // (list entries name its triangles' edges) and the list's capacity
    const float4* ray_soup[2] = {nullptr, nullptr};
    int64_t ray_bound[2] = {-1, -1};
    // rays from triangles: per group of ray_entry_group[d] soup triangles,
    // the four-wide target node its walks start at (group_entry)
    int32_t* ray_entry[2] = {nullptr, nullptr};
    int ray_entry_group[2] = {1, 1};
    // rays the launches of direction d index (list capacity or edge count)
    int64_t rays_of(int d) const { return ray_soup[d] ? ray_bound[d] : (int64_t)(d ? B->ne : A->ne); }
    // Whether side d takes its rays from its kept triangles.  Automatically:
    // always without dataset edges; after grouped culling, when the side
    // keeps fewer than half of its triangles.  A side that keeps most of them
    // (a dense join) traces its own edge list instead: the kept triangles'
    // edges repeat every edge two triangles of different groups share, and
    // in dense joins those repeats cost more raw hits than the finer culling
    // saves (measured on 40 sweep joins: 6.46 against 4.60 s on the densest,
    // with 965 M against 644 M raw hits; the tube and ellipsoid joins keep
    // 1.5-17 % per side and run faster on the kept triangles).
    bool triangle_rays(int d, bool grouped) const {
        const pierce_dataset* ds = d ? B : A;
        if (o.edge_source == PIERCE_EDGES_TRIANGLES) return true;
        if (o.edge_source == PIERCE_EDGES_DATASET) return false;
        if (ds->ne == 0) return ds->nt > 0;
        if (!grouped) return false;
        const int64_t kept = (d ? vb : va).num_tris;
        return 2 * kept < (int64_t)ds->nt;
    }
    // Ray lists of the sides that trace their kept triangles' edges: the
    // edges of the side's per-join soup, G triangles per group, listed group
    // by group; a side's groups are filtered against the other side's
    // per-join hierarchy unless `prefiltered[d]` (a culling round already
    // kept only the groups that meet it).
    // Each listed group's segments start their walks at the group's entry
    // node in the other side's four-wide hierarchy (group_entry), when that
    // hierarchy is not partitioned.
    int soup_ray_lists(const bool use[2], const int G[2], const bool prefiltered[2]) {
        const DevDataset* v[2] = {&va, &vb};
        const int slot[2] = {SLOT_LIST_AB, SLOT_LIST_BA}, eslot[2] = {SLOT_ENTRY_AB, SLOT_ENTRY_BA};
        for (int d = 0; d < 2; ++d) {
            if (!use[d]) continue;
            const DevDataset& src = *v[d];
            const DevDataset& other = *v[1 - d];
            const int64_t n = src.soup ? src.num_tris : 0;
            void* p = nullptr;
            if (int s = scratch(ctx, slot[d], 4 * (3 * (size_t)n + 64), &p)) return s;
            list[d] = static_cast<uint32_t*>(p);
            ray_entry[d] = nullptr;
            ray_entry_group[d] = std::max(G[d], 1);
            const bool entries = o.traversal == 0 && other.nodes4 && !other.part_roots && !other.root_is_leaf;
            if (entries) {
                void* pe = nullptr;
                if (int s = scratch(ctx, eslot[d], 4 * ((size_t)n / ray_entry_group[d] + 64), &pe)) return s;
                ray_entry[d] = static_cast<int32_t*>(pe);
            }
            // a split join lists its shard's segments only (containment is
            // split by B object instead: every candidate's rays are traced)
            const int si = rays_by_candidates ? 0 : shard_i(), sn = rays_by_candidates ? 1 : shard_n();
            if (int s = launch_soup_rays(ctx, src.soup, n, G[d], prefiltered[d] ? nullptr : &other,
                                         (d ? B : A)->d_obj_part, list[d], words + d, si, sn,
                                         entries ? other.nodes4 : nullptr, ray_entry[d]))
                return s;
            ray_soup[d] = src.soup;
            ray_bound[d] = 3 * n;
            listed[d] = true;
        }
        return PIERCE_OK;
    }
    uint8_t* active = nullptr;
    // words: [0] list count A->B, [1] list count B->A, [2] warp cursor,
    //        [3] deferred-test count, [4] exactly resolved key count,
    //        [5] active triangles of A, [6] active triangles of B, [7] active chunks (chunk
    //        hierarchy), [8] chunk count of a culling pass, [9] [10] active chunks of A, B
    unsigned long long* words = nullptr;
    // device views of A and B the kernels traverse (their own BVH, or the
    // per-join BVH over active triangles)
    DevDataset va{}, vb{};
    unsigned long long* amb_queue = nullptr;
    uint64_t amb_cap = 0;
    bool defer = true;
    uint8_t* chunk_flags = nullptr;
    uint32_t* chunk_list = nullptr;  // active chunk ids of the culling pass in flight
    // object hierarchies of the per-join path, and whether parity runs on
    // object pairs (both datasets store each object's triangles contiguously)
    DevDataset objA_{}, objB_{};
    bool object_parity = false;
    // containment: the parity table of B's first vertices in A (odd entries
    // are the candidate pairs), computed once per join
    uint64_t min_table_slots = 0;  // pair table size floor after a table that proved too small
    int groups_a_ = 0;  // A's per-join soup: triangles per group (0: not a grouped build)

    // LEARNED sizing of an overlap join, once its hierarchies exist: the
    // network's prediction is capped by 4 x the sampled incidence bound
    // (k_group_incidences: 1/64 of A's kept groups against B's kept
    // triangles) + 4096.  Objects far longer than their neighbours (tubes)
    // have boxes that meet nearly everything, which the network's features
    // cannot see; their kept groups are small.  A cap below the true count
    // costs only the two-pass rerun.
    int cap_learned_size() {
        void* pc = nullptr;
        if (int s = scratch(ctx, SLOT_AUX, 64, &pc)) return s;
        unsigned long long* d_count = static_cast<unsigned long long*>(pc) + 2;
        constexpr int kStep = 64;
        if (int s = launch_group_incidences(ctx, va.soup, va.num_tris, groups_a_, kStep, vb, d_count)) return s;
        int64_t n = 0;
        if (int s = host_value(ctx, d_count, 8, &n, "sampled incidences")) return s;
        const uint64_t cap = 4 * (uint64_t)n * kStep + 4096;
        if (cap < o.expected_pairs) o.expected_pairs = cap;
        return PIERCE_OK;
    }
    bool pairs_pending = false;    // containment: candidate pairs to test before any hierarchy is built

    // Containment from the candidate pairs directly (k_containment_pairs):
    // the odd parity pairs none of whose triangles meet.  *fallback: some
    // pair was too large to test this way (nothing is emitted then).
    int containment_by_pairs(pierce_result** out, bool* fallback) {
        *fallback = false;
        uint64_t cap = 8 * (uint64_t)std::max(B->num_objects, 1) + 16;
        uint64_t* ckeys = nullptr;
        uint64_t n = 0;
        const int b = timer.record();
        for (;;) {
            void* p = nullptr;
            if (int s = scratch(ctx, SLOT_BUILD_D, cap * 8, &p)) return s;
            ckeys = static_cast<uint64_t*>(p);
            void* pc = nullptr;
            if (int s = scratch(ctx, SLOT_AUX, 64, &pc)) return s;
            unsigned long long* d_count = static_cast<unsigned long long*>(pc);
            cudaMemsetAsync(d_count, 0, 16, ctx->stream);
            if (int s = launch_containment_pairs(ctx, cont_ptable, cont_par, cont_pslots, va, vb, ckeys, d_count, cap,
                                                 d_count + 1))
                return s;
            int64_t nf = 0, nv = 0;
            if (int s = host_value(ctx, d_count + 1, 8, &nf, "containment pairs left over")) return s;
            if (nf > 0) {
                *fallback = true;
                return PIERCE_OK;
            }
            if (int s = host_value(ctx, d_count, 8, &nv, "containment count")) return s;
            n = (uint64_t)nv;
            if (n <= cap) break;
            cap = n;
            st.retries++;
        }
        timer.span(b, timer.record(), &st.ms_edge_rays[1]);
        st.containment_pairs = n;
        st.containment_by_pairs = 1;
        pierce_result* r = new pierce_result();
        r->count = n;
        r->capacity = n;
        r->containment_count = n;
        if (int s = result_alloc(ctx, (void**)&r->d_pairs, std::max<uint64_t>(n, 1) * 8)) {
            delete r;
            return s;
        }
        const int tb = timer.record();
        if (n)
            if (int s = sort_u64_keys(ctx, ckeys, reinterpret_cast<uint64_t*>(r->d_pairs), (int64_t)n)) {
                pierce_result_destroy(r);
                return s;
            }
        timer.span(tb, timer.record(), &st.ms_dedup);
        if (int s = keys_to_pairs(ctx, reinterpret_cast<uint64_t*>(r->d_pairs), (int64_t)n)) {
            pierce_result_destroy(r);
            return s;
        }
        *out = r;
        return PIERCE_OK;
    }
    // shards: this join traces shard `shard_i` of `shard_n` (rays by list
    // position, parity rays by source object)
    int shard_i() const { return o.shard_count > 1 ? o.shard_index : 0; }
    int shard_n() const { return o.shard_count > 1 ? o.shard_count : 1; }
    int64_t shard_lo(int64_t n) const { return n * shard_i() / shard_n(); }
    int64_t shard_hi(int64_t n) const { return n * (shard_i() + 1) / shard_n(); }
    bool rays_by_candidates = false;  // containment split by B object: every shard traces all its candidates' rays
    uint64_t* cont_ptable = nullptr;
    uint32_t* cont_par = nullptr;
    uint64_t cont_pslots = 0;

    // Parity of B's first vertices against A into SLOT_CONT_PARITY (a full
    // table is enlarged and the parity rerun).
    int containment_parity() {
        uint64_t pslots = table_slots_for(8 * (uint64_t)std::max(B->num_objects, 1), 0.5);
        for (int attempt = 0;; ++attempt) {
            void* p = nullptr;
            if (int s = scratch(ctx, SLOT_CONT_PARITY, pslots * 12, &p)) return s;
            uint64_t* ptable = static_cast<uint64_t*>(p);
            uint32_t* par = reinterpret_cast<uint32_t*>(ptable + pslots);
            cudaMemsetAsync(ptable, 0xFF, pslots * 8, ctx->stream);
            cudaMemsetAsync(par, 0, pslots * 4, ctx->stream);
            const int b = timer.record();
            const int64_t lo = shard_lo(B->num_objects), hi = shard_hi(B->num_objects);
            if (object_parity) {
                if (int s = launch_parity_objects(ctx, vb, objA_, va, &gridA_, 1, ptable, par, pslots, lo, hi))
                    return s;
            } else if (int s = launch_parity(ctx, vb, va, 1, ptable, par, pslots, lo, hi)) {
                return s;
            }
            timer.span(b, timer.record(), &st.ms_parity[1]);
            uint32_t bits = 0;
            if (int s = read_device_error(ctx, &bits)) return s;
            if (bits & ERR_STACK_OVERFLOW) return set_error(PIERCE_ERR_STACK_OVERFLOW, "BVH traversal stack overflow");
            if (bits & ERR_HASH_FULL) {
                if (attempt >= std::max(o.max_retries, 4)) return set_error(PIERCE_ERR_HASH_FULL, "parity table full");
                pslots *= 4;
                st.retries++;
                continue;
            }
            cont_ptable = ptable;
            cont_par = par;
            cont_pslots = pslots;
            return PIERCE_OK;
        }
    }
    ColumnGrid gridA_{}, gridB_{};  // parity candidates of each side as a target

    // Column grids of both sides' object boxes (scratch slots meta/entries):
    // both counting passes, then the two sizes read back together.
    // Column grids of the sides that are parity targets.  A grid depends
    // only on its dataset's object boxes: the first eager join builds it into
    // memory the dataset keeps; a join graph (whose plan fixes every host
    // read) and a join short of memory use the context's scratch instead.
    int column_grids(bool side_a = true, bool side_b = true) {
        const DevDataset* v[2] = {&va, &vb};
        pierce_dataset* ds[2] = {A, B};
        const int meta_slot[2] = {SLOT_GRID_A, SLOT_GRID_B}, entries_slot[2] = {SLOT_GRID_A_ENTRIES, SLOT_GRID_B_ENTRIES};
        ColumnGrid* g[2] = {&gridA_, &gridB_};
        bool want[2] = {side_a, side_b};
        for (int sd = 0; sd < 2; ++sd)
            if (want[sd] && ds[sd]->grid_ready) {
                *g[sd] = ds[sd]->grid;
                want[sd] = false;
            }
        if (A == B && want[0] && want[1]) want[1] = false;  // one dataset on both sides: one grid
        void* pm[2] = {nullptr, nullptr};
        bool keep[2] = {false, false};
        const int32_t* total[2] = {nullptr, nullptr};
        for (int sd = 0; sd < 2; ++sd) {
            if (!want[sd]) continue;
            const size_t mb = column_grid_bytes(v[sd]->num_objects);
            if (!ctx->plan) {
                if (cudaMallocFromPoolAsync(&pm[sd], mb, ctx->pool, ctx->stream) == cudaSuccess) keep[sd] = true;
                else cudaGetLastError();
            }
            if (!keep[sd])
                if (int s = scratch(ctx, meta_slot[sd], mb, &pm[sd])) return s;
            if (int s = column_grid_count(ctx, *v[sd], pm[sd], &total[sd])) return s;
        }
        for (int sd = 0; sd < 2; ++sd) {
            if (!want[sd]) continue;
            int64_t n = 0;
            if (int s = host_value(ctx, total[sd], 4, &n, "column grid size")) return s;
            void* pe = nullptr;
            const size_t eb = 4 * (size_t)std::max<int64_t>(n, 1);
            if (keep[sd] && cudaMallocFromPoolAsync(&pe, eb, ctx->pool, ctx->stream) != cudaSuccess) {
                cudaGetLastError();
                pe = nullptr;
            }
            if (!pe) {
                // the grid stays with this join: copy its meta to scratch too
                if (keep[sd]) {
                    void* pm2 = nullptr;
                    const size_t mb = column_grid_bytes(v[sd]->num_objects);
                    if (int s = scratch(ctx, meta_slot[sd], mb, &pm2)) return s;
                    cudaMemcpyAsync(pm2, pm[sd], mb, cudaMemcpyDeviceToDevice, ctx->stream);
                    cudaFreeAsync(pm[sd], ctx->stream);
                    pm[sd] = pm2;
                    keep[sd] = false;
                }
                if (int s = scratch(ctx, entries_slot[sd], eb, &pe)) return s;
            }
            if (int s = column_grid_fill(ctx, *v[sd], pm[sd], (int32_t*)pe, g[sd])) return s;
            if (keep[sd]) {
                if (int s = check_cuda(cudaStreamSynchronize(ctx->stream), "column grid")) return s;
                ds[sd]->d_grid = pm[sd];
                ds[sd]->d_grid_entries = pe;
                ds[sd]->device_bytes += column_grid_bytes(v[sd]->num_objects) + eb;
                ds[sd]->grid = *g[sd];
                ds[sd]->grid_ready = 1;
            }
        }
        if (A == B && side_a && side_b) gridB_ = gridA_;
        return PIERCE_OK;
    }

    int prepare() {
        defer = o.defer_exact != 0;
        va = A->view();
        vb = B->view();
        void* p = nullptr;
        const size_t nobj_a = (size_t)std::max(A->num_objects, 1), nobj_b = (size_t)std::max(B->num_objects, 1);
        // words, object flags, then chunk flags (triangles A, B, edges A, B)
        const size_t chunks = (A->nt + 31) / 32 + (B->nt + 31) / 32 + (A->ne + 31) / 32 + (B->ne + 31) / 32 + 4;
        if (int s = scratch(ctx, SLOT_CULL, 128 + nobj_a + nobj_b + chunks, &p)) return s;
        words = static_cast<unsigned long long*>(p);
        active = static_cast<uint8_t*>(p) + 128;
        chunk_flags = active + nobj_a + nobj_b;
        if (o.cull_objects || o.active_bvh) {
            // chunk lists round up to whole chunks: 32 spare entries
            if (int s = scratch(ctx, SLOT_LIST_AB, 4 * (A->ne + 64), &p)) return s;
            list[0] = static_cast<uint32_t*>(p);
            if (int s = scratch(ctx, SLOT_LIST_BA, 4 * (B->ne + 64), &p)) return s;
            list[1] = static_cast<uint32_t*>(p);
        }
        const uint64_t rays_hint = std::max<uint64_t>(A->ne + B->ne, 3 * (A->nt + B->nt) / 2);
        amb_cap = std::min<uint64_t>(std::max<uint64_t>(rays_hint, 1024), 1ull << 24);
        if (int s = scratch(ctx, SLOT_AMB, 8 * amb_cap, &p)) return s;
        amb_queue = static_cast<unsigned long long*>(p);
        if (o.active_bvh) return prepare_active_bvh();
        return PIERCE_OK;
    }

    // BVH of one dataset's object boxes (degenerate triangles lo, hi, hi).
    // The hierarchy over ds's object boxes (degenerate triangles lo, hi, hi),
    // with its four-wide copy.  It depends only on the dataset, so the first
    // join builds it into memory the dataset keeps (freed with the dataset)
    // and later joins reuse it; where that memory cannot be had (or a graph
    // is being captured) it goes to the context's scratch for this join.
    int object_bvh(pierce_dataset* ds, int slot, int slot4, DevDataset* out) {
        if (ds->obj_hier_ready) {
            *out = ds->obj_hier;
            return PIERCE_OK;
        }
        const int64_t n = ds->num_objects;
        const size_t m = (size_t)std::max<int64_t>(n, 1);
        const size_t bytes = 16 * m + (48 + 64) * m + 256 + 8 * (size_t)ds->num_parts;
        const size_t bytes4 = sizeof(Node4) * m + 256;
        void* p = nullptr;
        bool keep = false;
        if (!capturing(ctx)) {
            if (cudaMallocFromPoolAsync(&p, bytes + bytes4, ctx->pool, ctx->stream) == cudaSuccess) keep = true;
            else cudaGetLastError();
        }
        if (!keep)
            if (int s = scratch(ctx, slot, bytes, &p)) return s;
        uint32_t* idx = static_cast<uint32_t*>(p);
        int32_t* t2o = reinterpret_cast<int32_t*>(idx + 3 * m);
        char* q = reinterpret_cast<char*>(t2o + m);
        q += (256 - ((uintptr_t)q & 255)) & 255;
        float4* soup = reinterpret_cast<float4*>(q);
        Node* nodes = reinterpret_cast<Node*>(soup + 3 * m);
        int2* roots = ds->num_parts ? reinterpret_cast<int2*>(nodes + m) : nullptr;
        if (int s = launch_object_pseudo_tris(ctx, (int32_t)n, idx, t2o)) return s;
        BvhShape shape;
        if (int s = build_lbvh(ctx, ds->d_obj_box, idx, t2o, nullptr, n, 1, soup, nodes, &shape, nullptr,
                               ds->d_obj_part, ds->num_parts, roots))
            return s;
        *out = DevDataset{};
        out->soup = soup;
        out->nodes = nodes;
        out->num_tris = n;
        out->root_is_leaf = shape.root_is_leaf;
        out->root_leaf_count = shape.root_leaf_count;
        out->obj_part = ds->d_obj_part;
        out->part_roots = roots;
        out->soup_boxes = 1;
        if (!keep) return wide_nodes(*out, shape.num_nodes, slot4, true);
        if (shape.num_nodes > 0 && !shape.root_is_leaf) {
            char* q4 = static_cast<char*>(p) + bytes;
            q4 += (256 - ((uintptr_t)q4 & 255)) & 255;
            Node4* n4 = reinterpret_cast<Node4*>(q4);
            if (int s = collapse4(ctx, nodes, (int64_t)shape.num_nodes, n4)) return s;
            out->nodes4 = n4;
        }
        // complete before another stream of another context reads it
        if (int s = check_cuda(cudaStreamSynchronize(ctx->stream), "object hierarchy")) return s;
        ds->d_obj_hier = p;
        ds->obj_hier = *out;
        ds->obj_hier_ready = 1;
        ds->device_bytes += bytes + bytes4;
        return PIERCE_OK;
    }

    // Per-join BVHs over the triangles that can take part in an overlap pair
    // (objects, then 32-triangle chunks, whose box meets a box of the other
    // side).  Exact: a segment lies in its object's and chunk's box, and so
    // does every target triangle.  Parity runs on object pairs over the
    // datasets' own triangles, or keeps every triangle (see below).
    int prepare_active_bvh() {
        const int b0 = timer.record();
        object_parity = A->contiguous && B->contiguous;
        if (o.predicate == PIERCE_CONTAINMENT && !o.include_overlap_pairs && object_parity) {
            // containment = parity(B in A) \ overlap: the odd-parity pairs
            // are tested directly (containment_by_pairs), which needs only
            // A's object hierarchy and column grid for the parity; the rest
            // is built only if some pair is too large for that
            if (int s = object_bvh(A, SLOT_OBJ_A, SLOT_NODES4_OBJ_A, &objA_)) return s;
            if (int s = column_grids(true, false)) return s;
            if (int s = containment_parity()) return s;
            rays_by_candidates = true;
            pairs_pending = true;
            timer.span(b0, timer.record(), &st.ms_build);
            return PIERCE_OK;
        }
        if (int s = object_bvh(A, SLOT_OBJ_A, SLOT_NODES4_OBJ_A, &objA_)) return s;
        if (int s = object_bvh(B, SLOT_OBJ_B, SLOT_NODES4_OBJ_B, &objB_)) return s;
        if (object_parity && o.predicate != PIERCE_OVERLAP)
            if (int s = column_grids()) return s;
        if (int s = launch_object_active(ctx, va, objB_, active)) return s;
        if (int s = launch_object_active(ctx, vb, objA_, active + std::max(A->num_objects, 1))) return s;
        return build_hierarchies(b0);
    }

    // Containment whose candidate pairs were too large to test directly:
    // B's object hierarchy, the object flags restricted to the candidates'
    // objects, then the culling pipeline.
    int containment_fallback() {
        const int b0 = timer.record();
        uint8_t* act_a = active;
        uint8_t* act_b = active + std::max(A->num_objects, 1);
        if (int s = object_bvh(B, SLOT_OBJ_B, SLOT_NODES4_OBJ_B, &objB_)) return s;
        if (int s = launch_object_active(ctx, va, objB_, act_a)) return s;
        if (int s = launch_object_active(ctx, vb, objA_, act_b)) return s;
        if (int s = launch_containment_candidates(ctx, cont_ptable, cont_par, cont_pslots, act_a, A->num_objects, act_b,
                                                  B->num_objects))
            return s;
        return build_hierarchies(b0);
    }

    // Culling rounds and per-join hierarchies (from the object flags
    // prepare_active_bvh computed).
    int build_hierarchies(int b0) {
        uint8_t* act_a = active;
        uint8_t* act_b = active + std::max(A->num_objects, 1);
        const DevDataset objA = objA_, objB = objB_;
        void *ta = nullptr, *tb = nullptr;
        if (int s = scratch(ctx, SLOT_TRIS_A, 4 * (A->nt + 64), &ta)) return s;
        if (int s = scratch(ctx, SLOT_TRIS_B, 4 * (B->nt + 64), &tb)) return s;
        void* pcl = nullptr;
        const size_t max_chunks = std::max((A->nt + 31) / 32, std::max((B->nt + 31) / 32,
                                           std::max((A->ne + 31) / 32, (B->ne + 31) / 32)));
        if (int s = scratch(ctx, SLOT_CHUNK_LIST, 4 * max_chunks + 64, &pcl)) return s;
        chunk_list = static_cast<uint32_t*>(pcl);
        // Chunk culling keeps the triangles and edges whose chunk box meets an
        // object box of the other side.  Parity (intersection, containment)
        // needs every triangle of a target object above the query point: it
        // runs on object pairs over the datasets' own triangles when their
        // objects are contiguous; otherwise the hierarchies keep whole objects.
        uint8_t* tchunk_a = chunk_flags;
        uint8_t* tchunk_b = tchunk_a + (A->nt + 31) / 32 + 1;
        uint8_t* echunk_a = tchunk_b + (B->nt + 31) / 32 + 1;
        uint8_t* echunk_b = echunk_a + (A->ne + 31) / 32 + 1;
        const bool chunked = o.cull_objects != 0;
        const bool tri_chunks = chunked && (o.predicate == PIERCE_OVERLAP || object_parity);
        const int leaf_a = join_leaf(o, A), leaf_b = join_leaf(o, B);
        // Chunk-culled sides build over groups of consecutive triangles (leaf
        // = one group of `leaf` triangles, rounded to a power of two).  In a
        // partitioned dataset no group may span two partitions (instanced
        // meshes never do); otherwise the hierarchies are built over the
        // surviving triangles.
        bool grouped = tri_chunks;
        if (grouped && A->num_parts > 0) {
            int32_t* mixed = reinterpret_cast<int32_t*>(words + 13);
            cudaMemsetAsync(mixed, 0, sizeof(int32_t), ctx->stream);
            if (int s = launch_group_mixed(ctx, nullptr, (int64_t)((A->nt + 31) / 32), A->d_tri_to_object,
                                           A->d_obj_part, (int64_t)A->nt, group_size(leaf_a), mixed))
                return s;
            if (int s = launch_group_mixed(ctx, nullptr, (int64_t)((B->nt + 31) / 32), B->d_tri_to_object,
                                           B->d_obj_part, (int64_t)B->nt, group_size(leaf_b), mixed))
                return s;
            int64_t m = 0;
            if (int s = host_value(ctx, mixed, 4, &m, "group partitions")) return s;
            grouped = m == 0;
        }
        if (grouped) {
            // 1. A's triangle chunks against B's object boxes; 2. A's per-join
            // hierarchy over the groups of those chunks that meet a B object
            // box; 3. B's chunks against A's kept triangles; 4. B's per-join
            // hierarchy over the groups of those chunks that meet one.  Groups
            // of a few consecutive triangles have tight boxes (a 32-triangle
            // chunk can straddle the ends of two tube branches), so B's
            // culling against A's kept triangles is much finer than against
            // boxes of A's chunks.  Every round keeps the triangles that
            // contain a point of the other side.
            if (int s = launch_chunk_cull(ctx, false, A->d_vertices, A->d_indices, A->d_tri_to_object, va, act_a, objB,
                                          tchunk_a, (uint32_t*)ta, words + 5, nullptr, chunk_list, words + 8))
                return s;
            bool filtered[2] = {false, false};
            if (int s = grouped_side(0, tchunk_a, (uint32_t*)ta, leaf_a, &objB_, &filtered[0])) return s;
            groups_a_ = group_size(leaf_a);
            if (int s = launch_chunk_cull(ctx, false, B->d_vertices, B->d_indices, B->d_tri_to_object, vb, act_b, va,
                                          tchunk_b, (uint32_t*)tb, words + 6, nullptr, chunk_list, words + 8))
                return s;
            if (int s = grouped_side(1, tchunk_b, (uint32_t*)tb, leaf_b, &va, &filtered[1])) return s;
            const bool use[2] = {triangle_rays(0, true), triangle_rays(1, true)};
            const int G[2] = {group_size(leaf_a), group_size(leaf_b)};
            // rays: A's groups against B's kept triangles; B's groups met A's already
            const bool pre[2] = {false, filtered[1]};
            if (int s = soup_ray_lists(use, G, pre)) return s;
            if (!use[0])
                if (int s = launch_chunk_cull(ctx, true, nullptr, nullptr, nullptr, va, act_a, vb, echunk_a, list[0],
                                              words + 0, nullptr, chunk_list, words + 8))
                    return s;
            if (!use[1])
                if (int s = launch_chunk_cull(ctx, true, nullptr, nullptr, nullptr, vb, act_b, va, echunk_b, list[1],
                                              words + 1, nullptr, chunk_list, words + 8))
                    return s;
            listed[0] = listed[1] = true;
            timer.span(b0, timer.record(), &st.ms_build);
            return PIERCE_OK;
        }
        if (tri_chunks) {
            // groups spanning partitions: the surviving chunks' triangles
            if (int s = launch_chunk_cull(ctx, false, A->d_vertices, A->d_indices, A->d_tri_to_object, va, act_a, objB,
                                          tchunk_a, (uint32_t*)ta, words + 5, nullptr, chunk_list, words + 8))
                return s;
            if (int s = launch_chunk_cull(ctx, false, B->d_vertices, B->d_indices, B->d_tri_to_object, vb, act_b, objA,
                                          tchunk_b, (uint32_t*)tb, words + 6, nullptr, chunk_list, words + 8))
                return s;
        } else {
            // Parity over these hierarchies counts every crossing above a first
            // vertex; for meshes that are not closed a crossing can come from
            // an object whose box the source's box does not meet, so the
            // parity predicates keep every triangle.  Overlap keeps the
            // triangles of active objects.
            const bool keep_all = o.predicate != PIERCE_OVERLAP;
            if (int s = launch_collect_tris(ctx, A->d_tri_to_object, (int64_t)A->nt, keep_all ? nullptr : act_a,
                                            (uint32_t*)ta, words + 5))
                return s;
            if (int s = launch_collect_tris(ctx, B->d_tri_to_object, (int64_t)B->nt, keep_all ? nullptr : act_b,
                                            (uint32_t*)tb, words + 6))
                return s;
        }
        const bool use_tri[2] = {triangle_rays(0, false), triangle_rays(1, false)};
        if (chunked) {
            if (!use_tri[0])
                if (int s = launch_chunk_cull(ctx, true, nullptr, nullptr, nullptr, va, act_a, objB, echunk_a,
                                              list[0], words + 0, nullptr, chunk_list, words + 8))
                    return s;
            if (!use_tri[1])
                if (int s = launch_chunk_cull(ctx, true, nullptr, nullptr, nullptr, vb, act_b, objA, echunk_b,
                                              list[1], words + 1, nullptr, chunk_list, words + 8))
                    return s;
        } else {
            if (!use_tri[0])
                if (int s = launch_collect_rays(ctx, va, act_a, list[0], words + 0)) return s;
            if (!use_tri[1])
                if (int s = launch_collect_rays(ctx, vb, act_b, list[1], words + 1)) return s;
        }
        listed[0] = listed[1] = true;
        int64_t na = 0, nb = 0;
        if (int s = host_value(ctx, words + 5, 8, &na, "active triangles of A")) return s;
        if (int s = host_value(ctx, words + 6, 8, &nb, "active triangles of B")) return s;
        void *sa = nullptr, *sb = nullptr, *na_p = nullptr, *nb_p = nullptr;
        if (int s = scratch(ctx, SLOT_RED_SOUP_A, 48 * (size_t)std::max<int64_t>(na, 1), &sa)) return s;
        const size_t roots_bytes = 8 * (size_t)A->num_parts;  // equal partition counts on both sides
        if (int s = scratch(ctx, SLOT_RED_NODES_A, 64 * (size_t)std::max<int64_t>(na, 1) + roots_bytes, &na_p))
            return s;
        if (int s = scratch(ctx, SLOT_RED_SOUP_B, 48 * (size_t)std::max<int64_t>(nb, 1), &sb)) return s;
        if (int s = scratch(ctx, SLOT_RED_NODES_B, 64 * (size_t)std::max<int64_t>(nb, 1) + roots_bytes, &nb_p))
            return s;
        int2* roots_a = A->num_parts ? reinterpret_cast<int2*>((Node*)na_p + std::max<int64_t>(na, 1)) : nullptr;
        int2* roots_b = B->num_parts ? reinterpret_cast<int2*>((Node*)nb_p + std::max<int64_t>(nb, 1)) : nullptr;
        BvhShape shA, shB;
        if (int s = build_lbvh(ctx, A->d_vertices, A->d_indices, A->d_tri_to_object, (const uint32_t*)ta, na,
                               leaf_a, (float4*)sa, (Node*)na_p, &shA, nullptr, A->d_obj_part, A->num_parts,
                               roots_a))
            return s;
        if (int s = build_lbvh(ctx, B->d_vertices, B->d_indices, B->d_tri_to_object, (const uint32_t*)tb, nb,
                               leaf_b, (float4*)sb, (Node*)nb_p, &shB, nullptr, B->d_obj_part, B->num_parts,
                               roots_b))
            return s;
        va.part_roots = roots_a;
        vb.part_roots = roots_b;
        va.soup = (const float4*)sa;
        va.nodes = (const Node*)na_p;
        va.num_tris = na;
        va.root_is_leaf = shA.root_is_leaf;
        va.root_leaf_count = shA.root_leaf_count;
        vb.soup = (const float4*)sb;
        vb.nodes = (const Node*)nb_p;
        vb.num_tris = nb;
        vb.root_is_leaf = shB.root_is_leaf;
        vb.root_leaf_count = shB.root_leaf_count;
        if (int s = wide_nodes(va, shA.num_nodes, SLOT_NODES4_A)) return s;
        if (int s = wide_nodes(vb, shB.num_nodes, SLOT_NODES4_B)) return s;
        {
            // the hierarchies hold the triangles of active objects: each
            // side's groups of 4 soup triangles against the other side's
            const int G[2] = {4, 4};
            const bool pre[2] = {false, false};
            // groups of soup triangles here may span partitions
            if (int s = soup_ray_lists(use_tri, G, pre)) return s;
        }
        st.active_triangles[0] = (uint64_t)na;
        st.active_triangles[1] = (uint64_t)nb;
        timer.span(b0, timer.record(), &st.ms_build);
        return PIERCE_OK;
    }

    // Four-wide copy of a hierarchy: per-join hierarchies for the
    // one-ray-per-thread walk (traversal 0; the other traversals walk the
    // binary nodes) and, always, the hierarchies that culling walks.
    int wide_nodes(DevDataset& v, uint64_t num_nodes, int slot, bool always = false) {
        v.nodes4 = nullptr;
        if ((o.traversal != 0 && !always) || num_nodes == 0 || v.root_is_leaf) return PIERCE_OK;
        void* p = nullptr;
        if (int s = scratch(ctx, slot, sizeof(Node4) * (size_t)num_nodes + 128, &p)) {
            // short of memory: the binary nodes serve every walk (slower)
            if (s != PIERCE_ERR_OUT_OF_MEMORY) return s;
            return PIERCE_OK;
        }
        // Node4 is 128-byte aligned; cudaMalloc returns 256-byte aligned memory
        if (int s = collapse4(ctx, v.nodes, (int64_t)num_nodes, static_cast<Node4*>(p))) return s;
        v.nodes4 = static_cast<const Node4*>(p);
        return PIERCE_OK;
    }

    // Per side: active chunk ids (into the side's triangle-list buffer), then
    // a hierarchy over groups of G consecutive triangles of those chunks.
    // triangles per group of a grouped build for leaf size `leaf`
    static int group_size(int leaf) {
        int g = 1;
        while (g < leaf && g < 32) g <<= 1;
        return g;
    }

    // One side's per-join hierarchy over groups of G consecutive triangles of
    // its flagged 32-triangle chunks (ids: the side's chunk-list buffer),
    // keeping only the groups whose box meets a leaf item of `filter` (a
    // four-wide hierarchy of the other side; none: every group).
    // *filtered tells whether the filter ran.
    int grouped_side(int sd, const uint8_t* flags, uint32_t* ids, int leaf, const DevDataset* filter, bool* filtered) {
        pierce_dataset* ds = sd ? B : A;
        const int G = group_size(leaf);
        const int64_t chunks = (int64_t)((ds->nt + 31) / 32);
        if (int s = launch_flag_list(ctx, flags, chunks, ids, words + 9 + sd)) return s;
        int64_t nc = 0;
        if (int s = host_value(ctx, words + 9 + sd, 8, &nc, "active chunks")) return s;
        const int64_t ng = nc * (32 / G);
        const int32_t parts = ds->num_parts;
        const int soup_slot = sd ? SLOT_RED_SOUP_B : SLOT_RED_SOUP_A, node_slot = sd ? SLOT_RED_NODES_B : SLOT_RED_NODES_A;
        void *sp = nullptr, *np = nullptr, *gp = nullptr;
        if (int s = scratch(ctx, soup_slot, 48 * 32 * (size_t)std::max<int64_t>(nc, 1), &sp)) return s;
        if (int s = scratch(ctx, node_slot, 64 * (size_t)std::max<int64_t>(ng, 1) + 8 * (size_t)parts, &np)) return s;
        int2* roots = parts ? reinterpret_cast<int2*>((Node*)np + std::max<int64_t>(ng, 1)) : nullptr;
        if (int s = scratch(ctx, SLOT_GROUPS, 96 * (size_t)std::max<int64_t>(ng, 1) + 512, &gp)) return s;
        if (filter && !filter->nodes4) filter = nullptr;
        *filtered = filter != nullptr;
        BvhShape sh;
        int64_t kept = ng;
        if (int s = build_grouped_lbvh(ctx, ds->d_vertices, ds->d_indices, ds->d_tri_to_object, (int64_t)ds->nt, ids,
                                       nc, G, gp, (float4*)sp, (Node*)np, &sh, filter, words + 11 + sd, &kept,
                                       ds->d_obj_part, parts, roots))
            return s;
        DevDataset& v = sd ? vb : va;
        v.soup = (const float4*)sp;
        v.nodes = (const Node*)np;
        v.num_tris = kept * G;
        v.root_is_leaf = sh.root_is_leaf;
        v.root_leaf_count = sh.root_leaf_count;
        v.part_roots = roots;
        // four-wide copy in every traversal mode: it also culls the other
        // side's chunks and filters its groups and rays
        if (int s = wide_nodes(v, sh.num_nodes, sd ? SLOT_NODES4_B : SLOT_NODES4_A, true)) return s;
        st.active_triangles[sd] = (uint64_t)(kept * G);
        return PIERCE_OK;
    }

    int precision_mode() const {
        if (o.precision == PIERCE_FP32) return 1;  // plain float32
        return defer ? 2 : 0;                      // deferred or inline exact
    }

    // Edge rays of the enabled directions.  COUNT and HASH queue undecided
    // tests and resolve them right away: into the table (HASH) or into
    // extra_keys (COUNT); WRITE skips them (already resolved by COUNT).
    int edge_rays(int mode, int32_t* counts_ab, int32_t* counts_ba, const int64_t* off_ab, const int64_t* off_ba,
                  uint64_t* keys, uint64_t* table, uint64_t slots, uint64_t* extra_keys = nullptr,
                  uint64_t extra_cap = 0) {
        const bool dirs[2] = {ab, ba};
        for (int d = 0; d < 2; ++d) {
            if (!dirs[d]) continue;
            const DevDataset& src = d ? vb : va;
            // the four-wide copies also serve culling; only traversal 0 walks them
            DevDataset tgt = d ? va : vb;
            if (o.traversal != 0) tgt.nodes4 = nullptr;
            int32_t* counts = d ? counts_ba : counts_ab;
            const int64_t* offs = d ? off_ba : off_ab;
            const int b = timer.record();
            RayOpts ro;
            if ((o.cull_objects || o.active_bvh) && (src.num_edges > 0 || ray_soup[d])) {
                if (!listed[d]) {
                    if (int s = launch_cull(ctx, src, tgt, active, list[d], words + d)) return s;
                    listed[d] = true;
                }
                ro.list = list[d];
                ro.count = words + d;
                ro.cursor = words + 2;
                ro.soup = ray_soup[d];
                ro.bound = rays_of(d);
                ro.entries = ray_entry[d];
                ro.entry_group = ray_entry_group[d];
                if (!rays_by_candidates) {
                    ro.shard_index = shard_i();
                    ro.shard_count = shard_n();
                }
                if (mode == 0) cudaMemsetAsync(counts, 0, 4 * (size_t)rays_of(d), ctx->stream);
            }
            if (!ro.list && !rays_by_candidates) {
                ro.shard_index = shard_i();
                ro.shard_count = shard_n();
            }
            ro.rays_per_fetch = o.rays_per_warp > 0 ? o.rays_per_warp : 32;
            ro.short_stack = o.stack_depth > 0 ? o.stack_depth : -1;
            ro.packets = o.traversal == 1 ? 1 : 0;
            const int prec = precision_mode();
            if (prec == 2) {
                ro.amb_queue = amb_queue;
                ro.amb_count = words + 3;
                ro.amb_cap = amb_cap;
                if (mode != 1) cudaMemsetAsync(words + 3, 0, 8, ctx->stream);
            }
            if (int s = launch_edge_rays(ctx, src, tgt, mode, prec, d, counts, offs, keys, table, slots, &ro))
                return s;
            if (prec == 2 && mode != 1)
                if (int s = launch_resolve(ctx, src, tgt, d, mode == 2 ? table : nullptr, slots, &ro, extra_keys,
                                           words + 4, extra_cap))
                    return s;
            timer.span(b, timer.record(), &st.ms_edge_rays[d]);
        }
        return PIERCE_OK;
    }

    // Overlap set in a hash table (scratch SLOT_TABLE); returns slots used.
    int overlap_hash(uint64_t** table_out, uint64_t* slots_out) {
        uint64_t slots;
        if (o.sizing == PIERCE_SIZING_FIXED && o.hash_table_slots > 0) {
            slots = 1;
            while (slots < o.hash_table_slots) slots <<= 1;
        } else {
            const uint64_t expected = o.expected_pairs ? o.expected_pairs : (8u << 20);
            slots = table_slots_for(expected, o.hash_load_factor);
        }
        while (slots < min_table_slots) slots <<= 1;
        for (int attempt = 0;; ++attempt) {
            void* p = nullptr;
            if (int s = scratch(ctx, SLOT_TABLE, slots * 8, &p)) return s;
            uint64_t* table = static_cast<uint64_t*>(p);
            cudaMemsetAsync(table, 0xFF, slots * 8, ctx->stream);
            if (int s = edge_rays(2, nullptr, nullptr, nullptr, nullptr, nullptr, table, slots)) return s;
            uint32_t bits = 0;
            if (int s = read_device_error(ctx, &bits)) return s;
            if (bits & ERR_STACK_OVERFLOW) return set_error(PIERCE_ERR_STACK_OVERFLOW, "BVH traversal stack overflow");
            if (bits & ERR_AMBIGUOUS_OVERFLOW) {
                defer = false;  // too many undecided tests to queue: resolve them inline
                continue;
            }
            if (bits & ERR_HASH_FULL) {
                if (attempt >= o.max_retries)
                    return set_error(PIERCE_ERR_HASH_FULL, "pair hash table full after retries");
                slots *= 4;
                st.retries++;
                continue;
            }
            *table_out = table;
            *slots_out = slots;
            st.hash_slots = slots;
            return PIERCE_OK;
        }
    }

    // Occupied slots of a table -> keys in SLOT_KEYS (at offset `base` keys);
    // the capacity is sized from the expected count and grown on overflow.
    int compact(const uint64_t* table, uint64_t slots, uint64_t base, uint64_t* n_out, uint64_t** keys_out) {
        uint64_t cap = o.expected_pairs ? (uint64_t)std::ceil((double)o.expected_pairs * std::max(1.0, o.output_safety))
                                        : (1u << 20);
        cap = std::max<uint64_t>(std::min<uint64_t>(cap, slots), 1024);
        for (int attempt = 0; attempt < 2; ++attempt) {
            void* p = nullptr;
            if (int s = scratch(ctx, SLOT_KEYS, (base + cap) * 8, &p)) return s;
            void* pc = nullptr;
            if (int s = scratch(ctx, SLOT_AUX, 64, &pc)) return s;
            unsigned long long* d_count = static_cast<unsigned long long*>(pc);
            cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), ctx->stream);
            uint64_t* keys = static_cast<uint64_t*>(p);
            if (int s = compact_table(ctx, table, slots, keys + base, cap, d_count)) return s;
            int64_t nv = 0;
            if (int s = host_value(ctx, d_count, 8, &nv, "compact count")) return s;
            const uint64_t n = (uint64_t)nv;
            st.result_capacity = cap;
            if (n <= cap) {
                *n_out = n;
                *keys_out = keys;
                return PIERCE_OK;
            }
            if (strict_capacity) return set_error(PIERCE_ERR_OUTPUT_OVERFLOW, "pairs exceed the predicted capacity");
            cap = n;  // output overflow: resize to the exact count and compact again
            st.retries++;
        }
        return set_error(PIERCE_ERR_OUTPUT_OVERFLOW, "compaction output overflow");
    }

    // Two-pass overlap: count, scan, write, sort + unique into SLOT_KEYS.
    int overlap_two_pass(uint64_t** keys_out, uint64_t* n_out) {
        const uint64_t na = ab ? (uint64_t)rays_of(0) : 0, nb = ba ? (uint64_t)rays_of(1) : 0;
        void* pc = nullptr;
        // counts (int32) and offsets (int64) for both directions
        const size_t cbytes = 4 * (na + nb) + 64, obytes = 8 * (na + nb) + 64;
        if (int s = scratch(ctx, SLOT_BUILD_A, cbytes, &pc)) return s;
        void* po = nullptr;
        if (int s = scratch(ctx, SLOT_BUILD_B, obytes, &po)) return s;
        int32_t* counts = static_cast<int32_t*>(pc);
        int64_t* offs = static_cast<int64_t*>(po);
        void* pe = nullptr;
        if (int s = scratch(ctx, SLOT_EXTRA, 8 * amb_cap, &pe)) return s;
        uint64_t* extra = static_cast<uint64_t*>(pe);
        const int64_t n_all = (int64_t)(na + nb);
        int64_t total = 0, total_ab = 0;
        uint64_t n_extra = 0;
        for (;;) {
            cudaMemsetAsync(words + 4, 0, 8, ctx->stream);
            // one zero count past the end: the scan's last offset is the total
            // (the last listed ray differs from run to run, the total does not)
            cudaMemsetAsync(counts + n_all, 0, 4, ctx->stream);
            const size_t span0 = timer.spans.size();
            if (int s = edge_rays(0, counts, counts + na, nullptr, nullptr, nullptr, nullptr, 0, extra, amb_cap))
                return s;
            // the pass-1 (count) spans also feed ms_count_pass
            const size_t span1 = timer.spans.size();
            for (size_t i = span0; i < span1; ++i) {
                double* target = timer.targets[i] == &st.ms_edge_rays[0] ? &st.ms_count_pass[0] : &st.ms_count_pass[1];
                timer.span(timer.spans[i].first, timer.spans[i].second, target);
            }
            int tb = timer.record();
            if (int s = exclusive_scan_i32_to_i64(ctx, counts, offs, n_all + 1)) return s;
            timer.span(tb, timer.record(), &st.ms_dedup);
            uint32_t bits = 0;
            if (int s = read_device_error(ctx, &bits)) return s;
            if (bits & ERR_STACK_OVERFLOW) return set_error(PIERCE_ERR_STACK_OVERFLOW, "BVH traversal stack overflow");
            if (bits & (ERR_AMBIGUOUS_OVERFLOW | ERR_OUTPUT_OVERFLOW)) {
                if (!defer) return set_error(PIERCE_ERR_OUTPUT_OVERFLOW, "resolved-test output overflow");
                defer = false;
                continue;
            }
            // total = last offset + last count; B->A offsets continue after the A total
            total = 0;
            int64_t off_b = 0, extra_n = 0;
            if (int s = host_value(ctx, offs + n_all, 8, &total, "scan total")) return s;
            if (na > 0 && nb > 0)
                if (int s = host_value(ctx, offs + na, 8, &off_b, "scan split")) return s;
            if (int s = host_value(ctx, words + 4, 8, &extra_n, "resolved keys")) return s;
            total_ab = (na > 0 && nb > 0) ? off_b : (na > 0 ? total : 0);
            n_extra = (uint64_t)extra_n;
            break;
        }
        st.raw_pairs[0] = (uint64_t)total_ab;
        st.raw_pairs[1] = (uint64_t)(total - total_ab);
        const int64_t n_raw = total + (int64_t)n_extra;
        // raw keys then sorted keys
        void* praw = nullptr;
        if (int s = scratch(ctx, SLOT_TABLE, 8 * (size_t)std::max<int64_t>(n_raw, 1), &praw)) return s;
        uint64_t* raw = static_cast<uint64_t*>(praw);
        if (int s = edge_rays(1, nullptr, nullptr, offs, offs + na, raw, nullptr, 0)) return s;
        if (n_extra) cudaMemcpyAsync(raw + total, extra, 8 * n_extra, cudaMemcpyDeviceToDevice, ctx->stream);
        void* pk = nullptr;
        if (int s = scratch(ctx, SLOT_KEYS, 8 * (size_t)std::max<int64_t>(n_raw, 1), &pk)) return s;
        uint64_t* sorted = static_cast<uint64_t*>(pk);
        int tb = timer.record();
        int64_t nu = 0;
        if (n_raw > 0) {
            if (int s = sort_u64_keys(ctx, raw, sorted, n_raw)) return s;
            if (int s = unique_u64(ctx, sorted, raw, n_raw, &nu)) return s;
            cudaMemcpyAsync(sorted, raw, 8 * (size_t)nu, cudaMemcpyDeviceToDevice, ctx->stream);
        }
        timer.span(tb, timer.record(), &st.ms_dedup);
        st.result_capacity = (uint64_t)n_raw;
        *keys_out = sorted;
        *n_out = (uint64_t)nu;
        return PIERCE_OK;
    }

    // Parity of src first vertices against tgt into the parity table, then
    // emit odd keys (mode 0: into out_table, mode 1: filtered append).
    int parity(const DevDataset& src, const DevDataset& tgt, int swap, double* ms, int emit_mode, uint64_t* out_table,
               uint64_t out_slots, const uint64_t* lookup_table, uint64_t lookup_slots, const uint64_t* lookup_sorted,
               int64_t lookup_n, uint64_t* out_keys, unsigned long long* out_count, uint64_t out_cap) {
        uint64_t pslots = table_slots_for(8 * (uint64_t)std::max(src.num_objects, 1), 0.5);
        for (int attempt = 0;; ++attempt) {
            void* p = nullptr;
            if (int s = scratch(ctx, SLOT_BUILD_C, pslots * 12, &p)) return s;
            uint64_t* ptable = static_cast<uint64_t*>(p);
            uint32_t* par = reinterpret_cast<uint32_t*>(ptable + pslots);
            cudaMemsetAsync(ptable, 0xFF, pslots * 8, ctx->stream);
            cudaMemsetAsync(par, 0, pslots * 4, ctx->stream);
            int b = timer.record();
            const int64_t lo = shard_lo(src.num_objects), hi = shard_hi(src.num_objects);
            if (object_parity) {
                if (int s = launch_parity_objects(ctx, src, swap ? objA_ : objB_, tgt, swap ? &gridA_ : &gridB_, swap,
                                                  ptable, par, pslots, lo, hi))
                    return s;
            } else if (int s = launch_parity(ctx, src, tgt, swap, ptable, par, pslots, lo, hi)) {
                return s;
            }
            timer.span(b, timer.record(), ms);
            uint32_t bits = 0;
            if (int s = read_device_error(ctx, &bits)) return s;
            if (bits & ERR_STACK_OVERFLOW) return set_error(PIERCE_ERR_STACK_OVERFLOW, "BVH traversal stack overflow");
            if (bits & ERR_HASH_FULL) {
                if (attempt >= o.max_retries) return set_error(PIERCE_ERR_HASH_FULL, "parity table full");
                pslots *= 4;
                st.retries++;
                continue;
            }
            if (int s = parity_emit(ctx, ptable, par, pslots, emit_mode, lookup_table, lookup_slots, lookup_sorted,
                                    lookup_n, out_table, out_slots, out_keys, out_count, out_cap))
                return s;
            return PIERCE_OK;
        }
    }

    // Parity of both directions into the pair table: both launches, one
    // error check, then both emits.  A full parity table falls back to one
    // direction at a time (each with its own enlarging retries).
    int parity_both(uint64_t* table, uint64_t slots) {
        const bool need[2] = {ab, ba};
        const int slot_of[2] = {SLOT_BUILD_C, SLOT_BUILD_D};
        uint64_t pslots[2] = {0, 0};
        uint64_t* ptable[2] = {nullptr, nullptr};
        uint32_t* par[2] = {nullptr, nullptr};
        for (int d = 0; d < 2; ++d) {
            if (!need[d]) continue;
            const DevDataset& src = d ? vb : va;
            const DevDataset& tgt = d ? va : vb;
            pslots[d] = table_slots_for(8 * (uint64_t)std::max(src.num_objects, 1), 0.5);
            void* p = nullptr;
            if (int s = scratch(ctx, slot_of[d], pslots[d] * 12, &p)) return s;
            ptable[d] = static_cast<uint64_t*>(p);
            par[d] = reinterpret_cast<uint32_t*>(ptable[d] + pslots[d]);
            cudaMemsetAsync(ptable[d], 0xFF, pslots[d] * 8, ctx->stream);
            cudaMemsetAsync(par[d], 0, pslots[d] * 4, ctx->stream);
            const int b = timer.record();
            const int64_t lo = shard_lo(src.num_objects), hi = shard_hi(src.num_objects);
            if (object_parity) {
                if (int s = launch_parity_objects(ctx, src, d ? objA_ : objB_, tgt, d ? &gridA_ : &gridB_, d,
                                                  ptable[d], par[d], pslots[d], lo, hi))
                    return s;
            } else if (int s = launch_parity(ctx, src, tgt, d, ptable[d], par[d], pslots[d], lo, hi)) {
                return s;
            }
            timer.span(b, timer.record(), &st.ms_parity[d]);
        }
        uint32_t bits = 0;
        if (int s = read_device_error(ctx, &bits)) return s;
        if (bits & ERR_STACK_OVERFLOW) return set_error(PIERCE_ERR_STACK_OVERFLOW, "BVH traversal stack overflow");
        if (bits & ERR_HASH_FULL) {
            st.retries++;
            for (int d = 0; d < 2; ++d)
                if (need[d])
                    if (int s = parity(d ? vb : va, d ? va : vb, d, &st.ms_parity[d], 0, table, slots, nullptr, 0,
                                       nullptr, 0, nullptr, nullptr, 0))
                        return s;
            return PIERCE_OK;
        }
        for (int d = 0; d < 2; ++d)
            if (need[d])
                if (int s = parity_emit(ctx, ptable[d], par[d], pslots[d], 0, nullptr, 0, nullptr, 0, table, slots,
                                        nullptr, nullptr, 0))
                    return s;
        return PIERCE_OK;
    }

    int make_result(const uint64_t* keys_sorted, uint64_t n, pierce_result** out) {
        pierce_result* r = new pierce_result();
        r->count = n;
        r->capacity = n;
        if (int s = result_alloc(ctx, (void**)&r->d_pairs, std::max<uint64_t>(n, 1) * sizeof(pierce_pair))) {
            delete r;
            return s;
        }
        if (n) {
            cudaMemcpyAsync(r->d_pairs, keys_sorted, n * 8, cudaMemcpyDeviceToDevice, ctx->stream);
            if (int s = keys_to_pairs(ctx, reinterpret_cast<uint64_t*>(r->d_pairs), (int64_t)n)) {
                pierce_result_destroy(r);
                return s;
            }
        }
        *out = r;
        return PIERCE_OK;
    }

    // Sort the keys in SLOT_KEYS[0..n) (unsorted, unique) into a result.
    int sort_into_result(uint64_t* keys, uint64_t n, pierce_result** out) {
        if (n == 0) return make_result(nullptr, 0, out);
        void* p = nullptr;
        if (int s = scratch(ctx, SLOT_BUILD_D, n * 8, &p)) return s;
        int tb = timer.record();
        if (int s = sort_u64_keys(ctx, keys, static_cast<uint64_t*>(p), (int64_t)n)) return s;
        timer.span(tb, timer.record(), &st.ms_dedup);
        return make_result(static_cast<uint64_t*>(p), n, out);
    }

    // Sort + unique keys[0..n) (may contain duplicates) into a result.
    int sort_unique_into_result(uint64_t* keys, uint64_t n, pierce_result** out) {
        if (n == 0) return make_result(nullptr, 0, out);
        void* p = nullptr;
        if (int s = scratch(ctx, SLOT_BUILD_D, n * 8, &p)) return s;
        int tb = timer.record();
        if (int s = sort_u64_keys(ctx, keys, static_cast<uint64_t*>(p), (int64_t)n)) return s;
        int64_t nu = 0;
        if (int s = unique_u64(ctx, static_cast<uint64_t*>(p), keys, (int64_t)n, &nu)) return s;
        timer.span(tb, timer.record(), &st.ms_dedup);
        return make_result(keys, (uint64_t)nu, out);
    }

    // LEARNED sizing: capacity = prediction x output_safety, no enlargement;
    // pairs that do not fit send the join to the two-pass method.
    bool strict_capacity = false;

    int run_predicate(pierce_result** out) {
        if (o.predicate == PIERCE_OVERLAP) return run_overlap(out);
        if (o.predicate == PIERCE_INTERSECTION) return run_intersection(out);
        return run_containment(out);
    }

    int run(pierce_result** out) {
        cudaMemsetAsync(ctx->d_counters, 0, sizeof(DevCounters), ctx->stream);
        cudaMemsetAsync(ctx->d_err, 0, sizeof(uint32_t), ctx->stream);
        const int t0 = timer.record();
        int s = PIERCE_OK;
        if (o.sizing == PIERCE_SIZING_LEARNED) {
            double log_pairs = 0.0;
            const int ts = timer.record();
            if ((s = learned_log_pairs(ctx, o.sizing_model, A, B, &log_pairs))) return s;
            timer.span(ts, timer.record(), &st.ms_sizing);
            // clamp: at most 2^31 expected pairs; a NaN prediction sizes the minimum table
            const double pred = std::isfinite(log_pairs) ? std::expm1(std::min(std::max(log_pairs, 0.0), 21.5)) : 0.0;
            st.predicted_pairs = pred;
            o.expected_pairs = std::max<uint64_t>((uint64_t)std::llround(pred), 1);
            o.sizing = PIERCE_SIZING_HASH;
            o.max_retries = 0;
            strict_capacity = true;
        }
        s = prepare();
        if (s) return s;
        if (strict_capacity && o.predicate == PIERCE_OVERLAP && groups_a_ > 0 && A->num_parts == 0)
            if ((s = cap_learned_size())) return s;
        s = run_predicate(out);
        if (strict_capacity && (s == PIERCE_ERR_HASH_FULL || s == PIERCE_ERR_OUTPUT_OVERFLOW)) {
            // the prediction was too small: the two-pass method sizes exactly
            st.sizing_overflow = 1;
            strict_capacity = false;
            o.sizing = PIERCE_SIZING_TWO_PASS;
            cudaMemsetAsync(ctx->d_err, 0, sizeof(uint32_t), ctx->stream);
            // the traversal counters describe the join that produced the pairs
            cudaMemsetAsync(ctx->d_counters, 0, sizeof(DevCounters), ctx->stream);
            s = run_predicate(out);
        }
        const int t1 = timer.record();
        timer.span(t0, t1, &st.ms_total);
        if (s) return s;
        cudaMemcpyAsync(ctx->h_counters, ctx->d_counters, sizeof(DevCounters), cudaMemcpyDeviceToHost, ctx->stream);
        if ((s = sync_ctx(ctx, "join"))) return s;
        timer.resolve();
        const DevCounters& c = *ctx->h_counters;
        st.rays = c.rays;
        st.node_visits = c.node_visits;
        st.tri_tests = c.tri_tests;
        st.raw_hits = c.raw_hits;
        st.fp32_ambiguous = c.fp32_ambiguous;
        st.fp64_ambiguous = c.fp64_ambiguous;
        st.parity_rays = c.parity_rays;
        st.hash_accesses = c.hash_accesses;
        st.hash_contentions = c.hash_contentions;
        st.num_pairs = (*out)->count;
        return PIERCE_OK;
    }

    int run_overlap(pierce_result** out) {
        if (o.sizing == PIERCE_SIZING_TWO_PASS) {
            uint64_t* keys = nullptr;
            uint64_t n = 0;
            if (int s = overlap_two_pass(&keys, &n)) return s;
            return make_result(keys, n, out);
        }
        uint64_t* table = nullptr;
        uint64_t slots = 0, n = 0;
        if (int s = overlap_hash(&table, &slots)) return s;
        uint64_t* keys = nullptr;
        int tb = timer.record();
        if (int s = compact(table, slots, 0, &n, &keys)) return s;
        timer.span(tb, timer.record(), &st.ms_dedup);
        return sort_into_result(keys, n, out);
    }

    int run_intersection(pierce_result** out) {
        if (o.sizing == PIERCE_SIZING_TWO_PASS) {
            uint64_t* okeys = nullptr;
            uint64_t n_over = 0;
            if (int s = overlap_two_pass(&okeys, &n_over)) return s;
            // parity keys are appended after the overlap keys, then sort + unique
            const uint64_t extra = (uint64_t)A->num_objects + (uint64_t)B->num_objects;
            void* p = nullptr;
            // move overlap keys to a buffer with room for the parity keys
            if (int s = scratch(ctx, SLOT_TABLE, (n_over + 8 * extra + 16) * 8, &p)) return s;
            uint64_t* all = static_cast<uint64_t*>(p);
            if (n_over) cudaMemcpyAsync(all, okeys, n_over * 8, cudaMemcpyDeviceToDevice, ctx->stream);
            void* pc = nullptr;
            if (int s = scratch(ctx, SLOT_AUX, 64, &pc)) return s;
            unsigned long long* d_count = static_cast<unsigned long long*>(pc);
            cudaMemsetAsync(d_count, 0, 8, ctx->stream);
            const uint64_t cap = 8 * extra + 16;
            if (ab)
                if (int s = parity(va, vb, 0, &st.ms_parity[0], 0, nullptr, 0, nullptr, 0, nullptr, 0, all + n_over,
                                   d_count, cap))
                    return s;
            if (ba)
                if (int s = parity(vb, va, 1, &st.ms_parity[1], 0, nullptr, 0, nullptr, 0, nullptr, 0, all + n_over,
                                   d_count, cap))
                    return s;
            int64_t n_par_v = 0;
            if (int s = host_value(ctx, d_count, 8, &n_par_v, "parity count")) return s;
            const uint64_t n_par = (uint64_t)n_par_v;
            if (n_par > cap) return set_error(PIERCE_ERR_OUTPUT_OVERFLOW, "parity output overflow");
            return sort_unique_into_result(all, n_over + n_par, out);
        }
        uint64_t* table = nullptr;
        uint64_t slots = 0, n = 0;
        for (int attempt = 0;; ++attempt) {
            if (int s = overlap_hash(&table, &slots)) return s;
            if (int s = parity_both(table, slots)) return s;
            uint32_t bits = 0;
            if (int s = read_device_error(ctx, &bits)) return s;
            if (!(bits & ERR_HASH_FULL)) break;
            // the parity pairs did not fit: a larger table, overlap and parity again
            if (attempt >= o.max_retries)
                return set_error(PIERCE_ERR_HASH_FULL, "pair table full while adding parity pairs");
            min_table_slots = 4 * slots;
            st.retries++;
        }
        uint64_t* keys = nullptr;
        int tb = timer.record();
        if (int s = compact(table, slots, 0, &n, &keys)) return s;
        timer.span(tb, timer.record(), &st.ms_dedup);
        return sort_into_result(keys, n, out);
    }

    int run_containment(pierce_result** out) {
        if (pairs_pending) {
            bool fallback = false;
            if (int s = containment_by_pairs(out, &fallback)) return s;
            if (!fallback) return PIERCE_OK;
            pairs_pending = false;
            if (int s = containment_fallback()) return s;
        }
        // Overlap set of A vs B (both directions as in the reference), then
        // parity of B's first vertices against A, filtered by the overlap set.
        const bool save_ab = ab, save_ba = ba;
        ab = ba = true;
        uint64_t* table = nullptr;
        uint64_t slots = 0;
        uint64_t* okeys = nullptr;
        uint64_t n_over = 0;
        const bool two_pass = o.sizing == PIERCE_SIZING_TWO_PASS;
        if (two_pass) {
            if (int s = overlap_two_pass(&okeys, &n_over)) return s;
        } else {
            if (int s = overlap_hash(&table, &slots)) return s;
        }
        ab = save_ab;
        ba = save_ba;
        if (!cont_ptable)
            if (int s = containment_parity()) return s;
        // odd parity pairs absent from the overlap set -> SLOT_BUILD_D (SLOT_TABLE
        // holds the hash table or the raw keys); a buffer that turns out too
        // small is enlarged to the count and the pairs emitted again
        uint64_t cap = 8 * (uint64_t)std::max(B->num_objects, 1) + 16;
        uint64_t* ckeys = nullptr;
        uint64_t n_cont = 0;
        for (;;) {
            void* p = nullptr;
            if (int s = scratch(ctx, SLOT_BUILD_D, cap * 8, &p)) return s;
            ckeys = static_cast<uint64_t*>(p);
            void* pc = nullptr;
            if (int s = scratch(ctx, SLOT_AUX, 64, &pc)) return s;
            unsigned long long* d_count = static_cast<unsigned long long*>(pc);
            cudaMemsetAsync(d_count, 0, 8, ctx->stream);
            if (int s = parity_emit(ctx, cont_ptable, cont_par, cont_pslots, 1, table, slots, okeys, (int64_t)n_over,
                                    nullptr, 0, ckeys, d_count, cap))
                return s;
            int64_t n_cont_v = 0;
            if (int s = host_value(ctx, d_count, 8, &n_cont_v, "containment count")) return s;
            n_cont = (uint64_t)n_cont_v;
            if (n_cont <= cap) break;
            cap = n_cont;
            st.retries++;
        }
        if (!two_pass && o.include_overlap_pairs) {
            // overlap keys of the table after the containment keys
            uint64_t* keys = nullptr;
            if (int s = compact(table, slots, 0, &n_over, &keys)) return s;
            okeys = keys;
        }
        st.containment_pairs = n_cont;
        st.overlap_pairs = n_over;
        // sort containment keys (into the front of a combined buffer)
        const uint64_t n_total = n_cont + (o.include_overlap_pairs ? n_over : 0);
        pierce_result* r = new pierce_result();
        r->count = n_total;
        r->capacity = n_total;
        r->containment_count = n_cont;
        if (int s = result_alloc(ctx, (void**)&r->d_pairs, std::max<uint64_t>(n_total, 1) * 8)) {
            delete r;
            return s;
        }
        uint64_t* rk = reinterpret_cast<uint64_t*>(r->d_pairs);
        int tb = timer.record();
        if (n_cont)
            if (int s = sort_u64_keys(ctx, ckeys, rk, (int64_t)n_cont)) {
                pierce_result_destroy(r);
                return s;
            }
        if (o.include_overlap_pairs && n_over) {
            if (two_pass) {
                cudaMemcpyAsync(rk + n_cont, okeys, n_over * 8, cudaMemcpyDeviceToDevice, ctx->stream);
            } else if (int s = sort_u64_keys(ctx, okeys, rk + n_cont, (int64_t)n_over)) {
                pierce_result_destroy(r);
                return s;
            }
        }
        timer.span(tb, timer.record(), &st.ms_dedup);
        if (int s = keys_to_pairs(ctx, rk, (int64_t)n_total)) {
            pierce_result_destroy(r);
            return s;
        }
        *out = r;
        return PIERCE_OK;
    }
};

}  // namespace

extern "C" {

}  // extern "C"

static int validate_join(pierce_ctx* ctx, pierce_dataset* a, pierce_dataset* b, const pierce_join_opts* opts,
                         pierce_join_opts* out_opts) {
    if ((!opts || !opts->active_bvh) && (!a->built || !b->built))
        return set_error(PIERCE_ERR_NOT_BUILT, "join: dataset not built (or use active_bvh)");
    if (a->ctx != ctx || b->ctx != ctx) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join: dataset of other ctx");
    if (a->num_parts != b->num_parts)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join: datasets have different partition counts");
    pierce_join_opts o;
    pierce_default_join_opts(&o);
    if (opts) o = *opts;
    if (o.predicate < 0 || o.predicate > 2 || o.direction < 0 || o.direction > 2 || o.sizing < 0 || o.sizing > 3 ||
        o.precision < 0 || o.precision > 1)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join: option out of range");
    if (o.sizing == PIERCE_SIZING_LEARNED && !o.sizing_model)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join: LEARNED sizing needs a sizing_model");
    if (!(o.hash_load_factor > 0.0 && o.hash_load_factor <= 1.0))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join: hash_load_factor must be in (0, 1]");
    if (o.leaf_size < 0 || o.leaf_size > 16 || o.rays_per_warp < 0 || o.rays_per_warp % 32 != 0 ||
        o.rays_per_warp > 1024 || o.stack_depth < 0 || o.stack_depth > 32 || o.traversal < 0 || o.traversal > 2)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join: tuning value out of range");
    if (o.edge_source < 0 || o.edge_source > 2)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join: edge_source out of range");
    const bool edgeless = (a->ne == 0 && a->nt > 0) || (b->ne == 0 && b->nt > 0);
    if (!o.active_bvh && (edgeless || o.edge_source == PIERCE_EDGES_TRIANGLES))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT,
                         "join: without active_bvh the rays are the datasets' edges (a dataset has none, or "
                         "edge_source asks for triangles)");
    if (o.edge_source == PIERCE_EDGES_DATASET && edgeless)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join: edge_source DATASET but a dataset has no edges");
    if (o.shard_count < 0 || o.shard_count > 65536 || o.shard_index < 0 ||
        (o.shard_count > 1 && o.shard_index >= o.shard_count) || (o.shard_count <= 1 && o.shard_index != 0))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join: shard_index must lie in [0, shard_count)");
    if (o.shard_count > 1 && o.predicate == PIERCE_CONTAINMENT &&
        (o.include_overlap_pairs || !o.active_bvh || !a->contiguous || !b->contiguous))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT,
                         "join: sharded containment splits by B object: it needs active_bvh, objects stored "
                         "contiguously and no include_overlap_pairs");
    *out_opts = o;
    return PIERCE_OK;
}

extern "C" {

int pierce_join(pierce_ctx* ctx, pierce_dataset* a, pierce_dataset* b, const pierce_join_opts* opts,
                pierce_result** out, pierce_stats* stats) {
    if (!ctx || !a || !b || !out) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join: null argument");
    *out = nullptr;
    pierce_join_opts o;
    if (int s = validate_join(ctx, a, b, opts, &o)) return s;
    cudaSetDevice(ctx->device);
    const uint64_t l0 = ctx->launches;
    Join j(ctx, a, b, o);
    int s = j.run(out);
    j.st.launches = (int32_t)(ctx->launches - l0);
    if (stats) *stats = j.st;
    return s;
}

int pierce_autotune_join(pierce_ctx* ctx, pierce_dataset* a, pierce_dataset* b, const pierce_join_opts* base,
                         int32_t repeats, pierce_tuned* best, pierce_tuned* trials, int32_t max_trials,
                         int32_t* num_trials) {
    if (!ctx || !a || !b || !best) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "autotune: null argument");
    pierce_join_opts o;
    if (int s = validate_join(ctx, a, b, base, &o)) return s;
    if (repeats < 1) repeats = 1;
    int32_t n_trials = 0;
    pierce_tuned cur;
    std::memset(&cur, 0, sizeof(cur));
    cur.leaf_size = join_leaf(o, a);
    cur.rays_per_warp = o.rays_per_warp > 0 ? o.rays_per_warp : 32;
    cur.stack_depth = o.stack_depth > 0 ? o.stack_depth : 8;
    cur.hash_load_factor = o.hash_load_factor;
    cur.traversal = o.traversal;
    cur.edge_source = o.edge_source;
    cur.ms = 1e300;
    // time one setting: one untimed run, then the best of `repeats`
    auto trial = [&](pierce_tuned& t) -> int {
        pierce_join_opts q = o;
        q.leaf_size = t.leaf_size;
        q.rays_per_warp = t.rays_per_warp;
        q.stack_depth = t.stack_depth;
        q.hash_load_factor = t.hash_load_factor;
        q.traversal = t.traversal;
        q.edge_source = t.edge_source;
        t.ms = 1e300;
        for (int r = 0; r <= repeats; ++r) {
            pierce_result* res = nullptr;
            pierce_stats st;
            if (int s = pierce_join(ctx, a, b, &q, &res, &st)) return s;
            pierce_result_destroy(res);
            if (r > 0) t.ms = std::min(t.ms, st.ms_total);
        }
        if (trials && n_trials < max_trials) trials[n_trials] = t;
        ++n_trials;
        return PIERCE_OK;
    };
    const bool hashed = o.sizing != PIERCE_SIZING_TWO_PASS;
    const std::vector<int> leaves = o.active_bvh ? std::vector<int>{1, 2, 4, 8} : std::vector<int>{cur.leaf_size};
    const std::vector<int> rays = {32, 64, 128}, stacks = {8, 16, 32};
    const std::vector<double> loads = hashed ? std::vector<double>{0.25, 0.5, 0.75}
                                             : std::vector<double>{cur.hash_load_factor};
    const std::vector<int> traversals = {0, 1, 2};
    // the rays' source: as given, or the datasets' edges when both hold them
    // (either gives the same pairs; which is faster depends on the meshes)
    std::vector<int> sources = {o.edge_source};
    if (o.edge_source != PIERCE_EDGES_DATASET && a->ne > 0 && b->ne > 0) sources.push_back(PIERCE_EDGES_DATASET);
    // coordinate descent: one parameter at a time, keeping the best so far
    for (int param = 0; param < 6; ++param) {
        const size_t n = param == 0 ? leaves.size() : param == 1 ? rays.size() : param == 2 ? stacks.size()
                         : param == 3 ? loads.size() : param == 4 ? traversals.size() : sources.size();
        pierce_tuned winner = cur;
        for (size_t i = 0; i < n; ++i) {
            pierce_tuned t = cur;
            if (param == 0) t.leaf_size = leaves[i];
            if (param == 1) t.rays_per_warp = rays[i];
            if (param == 2) t.stack_depth = stacks[i];
            if (param == 3) t.hash_load_factor = loads[i];
            if (param == 4) t.traversal = traversals[i];
            if (param == 5) t.edge_source = sources[i];
            if (int s = trial(t)) return s;
            if (t.ms < winner.ms) winner = t;
        }
        cur = winner;
    }
    *best = cur;
    if (num_trials) *num_trials = n_trials;
    return PIERCE_OK;
}

}  // extern "C"

// ---- joins captured as CUDA graphs -------------------------------------------

struct pierce_join_graph {
    pierce_ctx* ctx = nullptr;
    GraphPlan plan;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void* scratch[kScratchSlots] = {nullptr};  // the graph's own scratch buffers
    size_t scratch_bytes[kScratchSlots] = {0};
    pierce_pair* d_pairs = nullptr;
    uint64_t count = 0;
    uint64_t containment_count = 0;
    pierce_stats stats{};
    int launches = 0;  // kernels per replay
};

namespace {

// The graph's scratch goes back to its context where the context's slot is
// smaller (the context must outlive its graphs).
void free_graph(pierce_join_graph* g) {
    if (!g) return;
    if (g->ctx) cudaSetDevice(g->ctx->device);
    cudaDeviceSynchronize();
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    for (void* p : g->plan.buffers)
        if (p) cudaFree(p);
    for (int i = 0; i < kScratchSlots; ++i) {
        if (!g->scratch[i]) continue;
        if (g->ctx && g->ctx->scratch_bytes[i] < g->scratch_bytes[i]) {
            if (g->ctx->scratch[i]) cudaFree(g->ctx->scratch[i]);
            g->ctx->scratch[i] = g->scratch[i];
            g->ctx->scratch_bytes[i] = g->scratch_bytes[i];
        } else {
            cudaFree(g->scratch[i]);
        }
    }
    if (g->plan.h_check) cudaFreeHost(g->plan.h_check);
    delete g;
}

// Run `body` with the context's scratch buffers swapped for the graph's own
// (so later joins on the context cannot move memory a replay uses).
template <class F>
int with_graph_scratch(pierce_ctx* ctx, pierce_join_graph* g, F body) {
    void* saved[kScratchSlots];
    size_t saved_bytes[kScratchSlots];
    for (int i = 0; i < kScratchSlots; ++i) {
        saved[i] = ctx->scratch[i];
        saved_bytes[i] = ctx->scratch_bytes[i];
        ctx->scratch[i] = g->scratch[i];
        ctx->scratch_bytes[i] = g->scratch_bytes[i];
    }
    ctx->plan = &g->plan;
    const int s = body();
    ctx->plan = nullptr;
    for (int i = 0; i < kScratchSlots; ++i) {
        g->scratch[i] = ctx->scratch[i];
        g->scratch_bytes[i] = ctx->scratch_bytes[i];
        ctx->scratch[i] = saved[i];
        ctx->scratch_bytes[i] = saved_bytes[i];
    }
    return s;
}

}  // namespace

extern "C" {

int pierce_join_graph_create(pierce_ctx* ctx, pierce_dataset* a, pierce_dataset* b, const pierce_join_opts* opts,
                             pierce_join_graph** out, pierce_stats* stats) {
    if (!ctx || !a || !b || !out) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join_graph_create: null argument");
    *out = nullptr;
    pierce_join_opts o;
    if (int s = validate_join(ctx, a, b, opts, &o)) return s;
    cudaSetDevice(ctx->device);
    if (int s = sync_ctx(ctx, "join graph")) return s;
    pierce_join_graph* g = new pierce_join_graph();
    g->ctx = ctx;
    // the graph takes over the context's scratch buffers (no second copy)
    for (int i = 0; i < kScratchSlots; ++i) {
        g->scratch[i] = ctx->scratch[i];
        g->scratch_bytes[i] = ctx->scratch_bytes[i];
        ctx->scratch[i] = nullptr;
        ctx->scratch_bytes[i] = 0;
    }
    // 1. the planning run: an ordinary join that records its host decisions
    int s = with_graph_scratch(ctx, g, [&]() {
        g->plan.mode = 1;
        const uint64_t l0 = ctx->launches;
        Join j(ctx, a, b, o);
        pierce_result* r = nullptr;
        int st = j.run(&r);
        j.st.launches = (int32_t)(ctx->launches - l0);
        g->stats = j.st;
        if (st) return st;
        g->d_pairs = r->d_pairs;
        g->count = r->count;
        g->containment_count = r->containment_count;
        r->d_pairs = nullptr;  // the buffer belongs to the plan
        pierce_result_destroy(r);
        return (int)PIERCE_OK;
    });
    if (s == PIERCE_OK && !g->plan.values.empty()) {
        if (cudaHostAlloc((void**)&g->plan.h_check, 8 * g->plan.values.size(), cudaHostAllocDefault) != cudaSuccess)
            s = set_error(PIERCE_ERR_OUT_OF_MEMORY, "join graph: pinned check slots");
    }
    // 2. the same join under stream capture, taking the recorded decisions
    if (s == PIERCE_OK) {
        s = with_graph_scratch(ctx, g, [&]() {
            g->plan.mode = 2;
            g->plan.cursor = 0;
            g->plan.buf_cursor = 0;
            if (int e = check_cuda(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed), "begin capture"))
                return e;
            const uint64_t l0 = ctx->launches;
            Join j(ctx, a, b, o);
            pierce_result* r = nullptr;
            int st = j.run(&r);
            g->launches = (int)(ctx->launches - l0);
            cudaGraph_t graph = nullptr;
            const cudaError_t ec = cudaStreamEndCapture(ctx->stream, &graph);
            if (r) {
                r->d_pairs = nullptr;
                pierce_result_destroy(r);
            }
            if (st) {
                if (graph) cudaGraphDestroy(graph);
                return st;
            }
            if (int e = check_cuda(ec, "end capture")) return e;
            g->graph = graph;
            if (g->plan.cursor != g->plan.values.size())
                return set_error(PIERCE_ERR_CUDA, "join graph capture did not consume its plan");
            return check_cuda(cudaGraphInstantiate(&g->exec, graph, 0), "graph instantiate");
        });
    }
    if (s) {
        cudaGetLastError();
        free_graph(g);
        return s;
    }
    if (stats) *stats = g->stats;
    *out = g;
    return PIERCE_OK;
}

int pierce_join_graph_launch(pierce_ctx* ctx, pierce_join_graph* g, pierce_stats* stats) {
    if (!ctx || !g || g->ctx != ctx) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join_graph_launch: bad argument");
    cudaSetDevice(ctx->device);
    GraphPlan& p = g->plan;
    if (p.h_check) std::memset(p.h_check, 0, 8 * p.values.size());
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    cudaError_t e = cudaGraphLaunch(g->exec, ctx->stream);
    cudaEventRecord(e1, ctx->stream);
    int s = check_cuda(e, "graph launch");
    if (!s) s = check_cuda(cudaStreamSynchronize(ctx->stream), "graph replay");
    float ms = 0.0f;
    if (!s) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s) return s;
    ctx->launches += (uint64_t)g->launches;
    // the replay must have met every decision of the plan
    for (size_t i = 0; i < p.values.size(); ++i) {
        int64_t v = p.h_check[i];
        if (p.widths[i] == 4) {
            int32_t w;
            std::memcpy(&w, &p.h_check[i], 4);
            v = w;
        }
        if (v != p.values[i])
            return set_error(PIERCE_ERR_OUTPUT_OVERFLOW,
                             "join graph replay: a data-dependent size differs from the plan (inputs changed?)");
    }
    cudaMemcpy(ctx->h_err, ctx->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (*ctx->h_err) {
        const uint32_t bits = *ctx->h_err;
        cudaMemset(ctx->d_err, 0, sizeof(uint32_t));
        if (bits & ERR_STACK_OVERFLOW) return set_error(PIERCE_ERR_STACK_OVERFLOW, "BVH traversal stack overflow");
        if (bits & ERR_HASH_FULL) return set_error(PIERCE_ERR_HASH_FULL, "pair hash table full");
        return set_error(PIERCE_ERR_OUTPUT_OVERFLOW, "join graph replay: device capacity exceeded");
    }
    if (stats) {
        *stats = g->stats;
        const DevCounters& c = *ctx->h_counters;  // copied by the graph's last node
        stats->ms_total = ms;
        stats->rays = c.rays;
        stats->node_visits = c.node_visits;
        stats->tri_tests = c.tri_tests;
        stats->raw_hits = c.raw_hits;
        stats->fp32_ambiguous = c.fp32_ambiguous;
        stats->fp64_ambiguous = c.fp64_ambiguous;
        stats->parity_rays = c.parity_rays;
        stats->hash_accesses = c.hash_accesses;
        stats->hash_contentions = c.hash_contentions;
        stats->launches = g->launches;
        for (double* t : {&stats->ms_edge_rays[0], &stats->ms_edge_rays[1], &stats->ms_parity[0],
                          &stats->ms_parity[1], &stats->ms_dedup, &stats->ms_count_pass[0], &stats->ms_count_pass[1],
                          &stats->ms_build, &stats->ms_sizing})
            *t = 0.0;  // no per-phase events inside a replay
    }
    return PIERCE_OK;
}

int pierce_join_graph_pairs(const pierce_join_graph* g, const pierce_pair** d_pairs, uint64_t* count) {
    if (!g || !d_pairs || !count) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join_graph_pairs: null argument");
    *d_pairs = g->d_pairs;
    *count = g->count;
    return PIERCE_OK;
}

int pierce_join_graph_copy(pierce_ctx* ctx, const pierce_join_graph* g, pierce_pair* host_out, uint64_t capacity) {
    if (!ctx || !g || (!host_out && capacity)) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "join_graph_copy: null");
    const uint64_t n = std::min(capacity, g->count);
    if (n)
        if (int s = check_cuda(cudaMemcpyAsync(host_out, g->d_pairs, n * sizeof(pierce_pair), cudaMemcpyDeviceToHost,
                                               ctx->stream),
                               "graph result copy"))
            return s;
    if (int s = check_cuda(cudaStreamSynchronize(ctx->stream), "graph result copy")) return s;
    return g->count > capacity ? set_error(PIERCE_ERR_OUTPUT_OVERFLOW, "join_graph_copy: capacity below pair count")
                               : PIERCE_OK;
}

void pierce_join_graph_destroy(pierce_join_graph* g) { free_graph(g); }

int pierce_launch_edge_rays(pierce_ctx* ctx, const pierce_dataset* src, const pierce_dataset* tgt, int mode,
                            int precision, int swap, int32_t* d_counts, const int64_t* d_offsets, uint64_t* d_keys,
                            uint64_t* d_table, uint64_t table_slots, pierce_stats* stats) {
    if (!ctx || !src || !tgt) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "launch_edge_rays: null argument");
    if (!tgt->built) return set_error(PIERCE_ERR_NOT_BUILT, "launch_edge_rays: target not built");
    if (src->num_parts != tgt->num_parts)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "launch_edge_rays: datasets have different partition counts");
    if (mode == PIERCE_RAYS_COUNT && !d_counts) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "COUNT needs d_counts");
    if (mode == PIERCE_RAYS_WRITE && (!d_offsets || !d_keys))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "WRITE needs d_offsets and d_keys");
    if (mode == PIERCE_RAYS_HASH && (!d_table || table_slots == 0 || (table_slots & (table_slots - 1))))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "HASH needs a power-of-two table");
    cudaSetDevice(ctx->device);
    cudaMemsetAsync(ctx->d_counters, 0, sizeof(DevCounters), ctx->stream);
    if (int s = launch_edge_rays(ctx, src->view(), tgt->view(), mode, precision, swap, d_counts, d_offsets, d_keys,
                                 d_table, table_slots, nullptr))
        return s;
    uint32_t bits = 0;
    if (int s = read_device_error(ctx, &bits)) return s;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        cudaMemcpyAsync(ctx->h_counters, ctx->d_counters, sizeof(DevCounters), cudaMemcpyDeviceToHost, ctx->stream);
        if (int s = sync_ctx(ctx, "counters")) return s;
        stats->rays = ctx->h_counters->rays;
        stats->node_visits = ctx->h_counters->node_visits;
        stats->tri_tests = ctx->h_counters->tri_tests;
        stats->raw_hits = ctx->h_counters->raw_hits;
        stats->fp32_ambiguous = ctx->h_counters->fp32_ambiguous;
        stats->fp64_ambiguous = ctx->h_counters->fp64_ambiguous;
    }
    if (bits & ERR_STACK_OVERFLOW) return set_error(PIERCE_ERR_STACK_OVERFLOW, "BVH traversal stack overflow");
    if (bits & ERR_HASH_FULL) return set_error(PIERCE_ERR_HASH_FULL, "hash table full");
    return PIERCE_OK;
}

int pierce_launch_parity(pierce_ctx* ctx, const pierce_dataset* src, const pierce_dataset* tgt, int precision,
                         int swap, uint64_t* d_table, uint32_t* d_parity, uint64_t table_slots, pierce_stats* stats) {
    (void)precision;
    if (!ctx || !src || !tgt || !d_table || !d_parity || table_slots == 0 || (table_slots & (table_slots - 1)))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "launch_parity: bad argument");
    if (!tgt->built) return set_error(PIERCE_ERR_NOT_BUILT, "launch_parity: target not built");
    if (src->num_parts != tgt->num_parts)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "launch_parity: datasets have different partition counts");
    cudaSetDevice(ctx->device);
    cudaMemsetAsync(ctx->d_counters, 0, sizeof(DevCounters), ctx->stream);
    if (int s = launch_parity(ctx, src->view(), tgt->view(), swap, d_table, d_parity, table_slots)) return s;
    uint32_t bits = 0;
    if (int s = read_device_error(ctx, &bits)) return s;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        cudaMemcpyAsync(ctx->h_counters, ctx->d_counters, sizeof(DevCounters), cudaMemcpyDeviceToHost, ctx->stream);
        if (int s = sync_ctx(ctx, "counters")) return s;
        stats->parity_rays = ctx->h_counters->parity_rays;
        stats->node_visits = ctx->h_counters->node_visits;
        stats->tri_tests = ctx->h_counters->tri_tests;
    }
    if (bits & ERR_STACK_OVERFLOW) return set_error(PIERCE_ERR_STACK_OVERFLOW, "BVH traversal stack overflow");
    if (bits & ERR_HASH_FULL) return set_error(PIERCE_ERR_HASH_FULL, "parity table full");
    return PIERCE_OK;
}

int pierce_parity_tracking(pierce_ctx* ctx, const pierce_dataset* src, const pierce_dataset* tgt, int32_t max_targets,
                           int32_t* target_ids, uint32_t* target_hits, uint32_t* targets_crossed,
                           uint32_t* overflows) {
    if (!ctx || !src || !tgt || max_targets < 1 || max_targets > (1 << 16))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "parity_tracking: bad argument");
    if (src->num_parts != tgt->num_parts)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "parity_tracking: datasets have different partition counts");
    if (tgt->num_objects > 0 && !tgt->contiguous)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT,
                         "parity_tracking: the target's objects do not store their triangles contiguously");
    const int64_t n = src->num_objects;
    if (n <= 0) return PIERCE_OK;
    cudaSetDevice(ctx->device);
    ++ctx->scratch_gen;
    const DevDataset vs = src->view(), vt = tgt->view();
    // candidates: the column grid of the target's object boxes
    void* meta = nullptr;
    if (int s = scratch(ctx, SLOT_GRID_B, column_grid_bytes(tgt->num_objects), &meta)) return s;
    const int32_t* d_total = nullptr;
    if (int s = column_grid_count(ctx, vt, meta, &d_total)) return s;
    int64_t entries = 0;
    if (int s = host_value(ctx, d_total, 4, &entries, "column grid size")) return s;
    void* pe = nullptr;
    if (int s = scratch(ctx, SLOT_GRID_B_ENTRIES, 4 * (size_t)std::max<int64_t>(entries, 1), &pe)) return s;
    ColumnGrid grid{};
    if (int s = column_grid_fill(ctx, vt, meta, static_cast<int32_t*>(pe), &grid)) return s;
    // ids and hits (max_targets slots per source object), then crossed and overflow
    const size_t slots = (size_t)n * (size_t)max_targets;
    void* d = nullptr;
    if (int s = device_alloc(&d, 8 * slots + 8 * (size_t)n, "parity tracking")) return s;
    int32_t* ids = static_cast<int32_t*>(d);
    uint32_t* hits = reinterpret_cast<uint32_t*>(ids + slots);
    uint32_t* crossed = hits + slots;
    uint32_t* overflow = crossed + n;
    cudaStream_t st = ctx->stream;
    int s = check_cuda(cudaMemsetAsync(ids, 0xFF, 4 * slots, st), "parity tracking");
    if (!s) s = check_cuda(cudaMemsetAsync(hits, 0, 4 * slots + 8 * (size_t)n, st), "parity tracking");
    if (!s) s = launch_parity_tracking(ctx, vs, vt, grid, max_targets, ids, hits, crossed, overflow);
    if (!s && target_ids)
        s = check_cuda(cudaMemcpyAsync(target_ids, ids, 4 * slots, cudaMemcpyDeviceToHost, st), "parity tracking");
    if (!s && target_hits)
        s = check_cuda(cudaMemcpyAsync(target_hits, hits, 4 * slots, cudaMemcpyDeviceToHost, st), "parity tracking");
    if (!s && targets_crossed)
        s = check_cuda(cudaMemcpyAsync(targets_crossed, crossed, 4 * (size_t)n, cudaMemcpyDeviceToHost, st),
                       "parity tracking");
    if (!s && overflows)
        s = check_cuda(cudaMemcpyAsync(overflows, overflow, 4 * (size_t)n, cudaMemcpyDeviceToHost, st),
                       "parity tracking");
    uint32_t bits = 0;
    if (!s) s = read_device_error(ctx, &bits);  // synchronises the stream
    cudaStreamSynchronize(st);
    cudaFree(d);
    if (s) return s;
    if (bits & ERR_STACK_OVERFLOW) return set_error(PIERCE_ERR_STACK_OVERFLOW, "BVH traversal stack overflow");
    return PIERCE_OK;
}

int pierce_exclusive_scan(pierce_ctx* ctx, const int32_t* d_counts, int64_t* d_offsets, int64_t n, int64_t* total) {
    if (!ctx || (n > 0 && (!d_counts || !d_offsets)) || !total)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "exclusive_scan: bad argument");
    cudaSetDevice(ctx->device);
    *total = 0;
    if (n <= 0) return PIERCE_OK;
    if (int s = exclusive_scan_i32_to_i64(ctx, d_counts, d_offsets, n)) return s;
    cudaMemcpyAsync(ctx->h_small, d_offsets + n - 1, 8, cudaMemcpyDeviceToHost, ctx->stream);
    cudaMemcpyAsync(ctx->h_small + 1, d_counts + n - 1, 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (int s = sync_ctx(ctx, "scan total")) return s;
    *total = ctx->h_small[0] + (int64_t)(int32_t)(ctx->h_small[1] & 0xFFFFFFFF);
    return PIERCE_OK;
}

int pierce_merge_and_deduplicate_pairs(pierce_ctx* ctx, const pierce_pair* d1, int64_t n1, const pierce_pair* d2,
                                       int64_t n2, pierce_pair* d_out, int64_t* num_unique) {
    if (!ctx || !num_unique || n1 < 0 || n2 < 0 || (n1 && !d1) || (n2 && !d2) || ((n1 + n2) && !d_out))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "merge_and_deduplicate: bad argument");
    cudaSetDevice(ctx->device);
    *num_unique = 0;
    const int64_t n = n1 + n2;
    if (n == 0) return PIERCE_OK;
    void *pa = nullptr, *pb = nullptr;
    if (int s = scratch(ctx, SLOT_KEYS, 8 * (size_t)n, &pa)) return s;
    if (int s = scratch(ctx, SLOT_BUILD_D, 8 * (size_t)n, &pb)) return s;
    uint64_t* keys = static_cast<uint64_t*>(pa);
    uint64_t* sorted = static_cast<uint64_t*>(pb);
    if (n1) pairs_to_keys(ctx, reinterpret_cast<const uint64_t*>(d1), keys, n1);
    if (n2) pairs_to_keys(ctx, reinterpret_cast<const uint64_t*>(d2), keys + n1, n2);
    if (int s = sort_u64_keys(ctx, keys, sorted, n)) return s;
    int64_t nu = 0;
    if (int s = unique_u64(ctx, sorted, keys, n, &nu)) return s;
    if (int s = keys_to_pairs(ctx, keys, nu)) return s;
    cudaMemcpyAsync(d_out, keys, 8 * (size_t)nu, cudaMemcpyDeviceToDevice, ctx->stream);
    if (int s = sync_ctx(ctx, "merge_and_deduplicate")) return s;
    *num_unique = nu;
    return PIERCE_OK;
}

int pierce_compact_hash_table_pairs(pierce_ctx* ctx, const uint64_t* d_table, uint64_t table_slots, pierce_pair* d_out,
                                    uint64_t max_output, uint64_t* count) {
    if (!ctx || !d_table || !count || (max_output && !d_out))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "compact_hash_table_pairs: bad argument");
    cudaSetDevice(ctx->device);
    void* pc = nullptr;
    if (int s = scratch(ctx, SLOT_AUX, 64, &pc)) return s;
    unsigned long long* d_count = static_cast<unsigned long long*>(pc);
    cudaMemsetAsync(d_count, 0, 8, ctx->stream);
    uint64_t* out = reinterpret_cast<uint64_t*>(d_out);
    if (int s = compact_table(ctx, d_table, table_slots, out, max_output, d_count)) return s;
    cudaMemcpyAsync(ctx->h_small, d_count, 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (int s = sync_ctx(ctx, "compact")) return s;
    *count = (uint64_t)ctx->h_small[0];
    const uint64_t n = std::min(*count, max_output);
    if (int s = keys_to_pairs(ctx, out, (int64_t)n)) return s;
    if (int s = sync_ctx(ctx, "compact")) return s;
    if (*count > max_output)
        return set_error(PIERCE_ERR_OUTPUT_OVERFLOW, "compact_hash_table_pairs: more pairs than max_output");
    return PIERCE_OK;
}

int pierce_estimate_pairs(pierce_ctx* ctx, const void* cells_a, uint32_t num_a, const void* cells_b, uint32_t num_b,
                          float cell_size, float epsilon, float gamma, int alpha_correction, double* raw,
                          int64_t* estimate, int32_t* matched_cells) {
    if (!ctx || (num_a && !cells_a) || (num_b && !cells_b) || !raw || !estimate)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "estimate_pairs: bad argument");
    struct Cell {
        int32_t ix, iy, iz;
        uint32_t center, touch;
        float size, ratio;
    };
    static_assert(sizeof(Cell) == 28, "cell layout");
    const Cell* A = static_cast<const Cell*>(cells_a);
    const Cell* B = static_cast<const Cell*>(cells_b);
    // match cells of B against A by index
    struct H {
        size_t operator()(uint64_t k) const { return std::hash<uint64_t>()(k * 0x9E3779B97F4A7C15ULL); }
    };
    auto key = [](const Cell& c) {
        return ((uint64_t)(uint32_t)c.ix * 0x100000001B3ULL) ^ ((uint64_t)(uint32_t)c.iy << 21) ^
               ((uint64_t)(uint32_t)c.iz << 42);
    };
    std::unordered_multimap<uint64_t, uint32_t, H> map;
    map.reserve(num_a * 2 + 1);
    for (uint32_t i = 0; i < num_a; ++i) map.emplace(key(A[i]), i);
    std::vector<Cell> ma, mb;
    for (uint32_t i = 0; i < num_b; ++i) {
        auto range = map.equal_range(key(B[i]));
        for (auto it = range.first; it != range.second; ++it) {
            const Cell& a = A[it->second];
            if (a.ix == B[i].ix && a.iy == B[i].iy && a.iz == B[i].iz) {
                ma.push_back(a);
                mb.push_back(B[i]);
                break;
            }
        }
    }
    float cell_volume = cell_size * cell_size * cell_size;
    double total = 0.0;
    if (!ma.empty())
        if (int s = estimate_cells(ctx, ma.data(), mb.data(), (int)ma.size(), cell_volume, epsilon, gamma, &total))
            return s;
    // global average size / volume ratio weighted by touch counts
    auto avg = [](const Cell* c, uint32_t n, bool ratio) {
        double sum = 0.0;
        long long cnt = 0;
        for (uint32_t i = 0; i < n; ++i)
            if (c[i].touch > 0) {
                sum += (double)(ratio ? c[i].ratio : c[i].size) * (double)c[i].touch;
                cnt += c[i].touch;
            }
        if (cnt == 0) return ratio ? 1.0f : 0.0f;
        return (float)(sum / cnt);
    };
    const float eff_a = avg(A, num_a, false) * std::cbrt(avg(A, num_a, true));
    const float eff_b = avg(B, num_b, false) * std::cbrt(avg(B, num_b, true));
    const float comb = eff_a + eff_b;
    const float mink = comb * comb * comb;
    if (cell_volume < 1e-9f) cell_volume = 1e-9f;
    float alpha = 1.0f;
    if (alpha_correction) {
        alpha = mink / cell_volume;
        if (alpha < 1.0f) alpha = 1.0f;
    }
    *raw = total;
    *estimate = (int64_t)((float)total / alpha);
    if (matched_cells) *matched_cells = (int32_t)ma.size();
    return PIERCE_OK;
}

}  // extern "C"
