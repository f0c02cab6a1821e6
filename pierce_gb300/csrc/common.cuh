// Shared device/host definitions of the GB300 join library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/pierce_capi.h"

namespace pgpu {

// Device-side error bits, OR-ed into one word per context and translated to
// pierce_status codes by the host after each join phase.
enum ErrBits : uint32_t {
    ERR_HASH_FULL = 1u,
    ERR_STACK_OVERFLOW = 2u,
    ERR_OUTPUT_OVERFLOW = 4u,
    ERR_QUEUE_TIMEOUT = 8u,
    ERR_AMBIGUOUS_OVERFLOW = 16u,  // deferred-test queue full: rerun with inline exact tests
};

constexpr uint64_t kEmptyKey = 0xFFFFFFFFFFFFFFFFull;
constexpr int kStackSize = 64;  // >= depth of any LBVH over 30-bit Morton + index keys
// a Node4 walk pushes at most 3 entries per Node4 level, half as many levels
constexpr int kStackSize4 = 96;

// Counters accumulated by traversal kernels (one atomicAdd per warp).
struct DevCounters {
    unsigned long long rays;
    unsigned long long node_visits;
    unsigned long long tri_tests;
    unsigned long long raw_hits;
    unsigned long long fp32_ambiguous;
    unsigned long long fp64_ambiguous;
    unsigned long long parity_rays;
    unsigned long long hash_accesses;
    unsigned long long hash_contentions;
    unsigned long long pad;
};

// Binary BVH node holding the boxes of its two children (64 bytes, four
// 16-byte vector loads).  Child encoding: c >= 0 internal node index,
// c < 0 leaf whose triangles are soup[~c .. ~c + count).
struct __align__(16) Node {
    float4 bx;   // c0.lo.x, c0.hi.x, c1.lo.x, c1.hi.x
    float4 by;   // c0.lo.y, c0.hi.y, c1.lo.y, c1.hi.y
    float4 bz;   // c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z
    int4 ch;     // child0, child1, leaf counts (count0 | count1 << 8),
                 // build link (parent << 2 | side << 1 | arrival toggle)
};

// Four-wide node collapsed from a binary hierarchy: Node4[n] holds the
// (up to) four grandchildren of binary internal node n, where a child that
// is a leaf stands for itself.  Node4 indices are binary node indices, so a
// traversal entering internal node c reads Node4[c] and skips a level: half
// the dependent node loads of the binary walk, one 128-byte line each.
// Unused entries have an empty box (lo > hi).
struct __align__(128) Node4 {
    float4 lox, hix, loy, hiy, loz, hiz;  // entry j: (lo.x, hi.x, ...)[j]
    int4 ch;                              // >= 0 internal node index, < 0 leaf ~first
    int4 meta;                            // x: leaf counts, 8 bits per entry
};

// Device view of one dataset (all pointers into its own allocations).
struct DevDataset {
    // triangle soup in BVH leaf order: per triangle 3 float4:
    //   (v0.xyz, object id bits), (v1.xyz, original triangle index bits), (v2.xyz, 0)
    const float4* soup;
    const Node* nodes;
    const Node4* nodes4;    // optional four-wide copy of nodes (per-join hierarchies)
    int64_t num_tris;
    int root_is_leaf;       // 1 when the whole dataset is a single leaf
    int root_leaf_count;
    // edge rays, 2 float4 per edge: (start.xyz, src object bits), (end.xyz, 0)
    const float4* edges;
    const int32_t* edge_src;     // source object per edge (compact copy)
    int64_t num_edges;
    // objects
    const float4* first_vertex;  // per object (xyz, 0)
    const float* obj_box;        // per object 6 floats lo.xyz hi.xyz
    int32_t num_objects;
    // partitioned datasets (a batch of independent joins): partition of each
    // object, and per partition the traversal start of this hierarchy
    // (x >= 0 internal node; x < 0 leaf ~x of y triangles; (-1, 0) empty)
    const int32_t* obj_part;
    const int2* part_roots;
    // the dataset's own triangles (parity by object pairs): vertices, indices
    // and per object its contiguous triangle range (first, count)
    const float* verts;
    const uint32_t* idx;
    const int2* obj_range;
    // boxes (lo.xyz, hi.xyz) of every 32 consecutive triangles / edges
    const float* tri_chunk_box;
    const float* edge_chunk_box;
    int edges_grouped;  // edges stored grouped by source object
    int soup_boxes;     // the soup holds boxes as degenerate triangles (lo, hi, hi), not triangles
};

// Optional inputs of an edge-ray launch: a compacted ray list (object
// culling) and the queue of deferred exact tests.
struct RayOpts {
    const uint32_t* list = nullptr;
    const unsigned long long* count = nullptr;
    unsigned long long* cursor = nullptr;
    unsigned long long* amb_queue = nullptr;
    unsigned long long* amb_count = nullptr;
    uint64_t amb_cap = 0;
    int rays_per_fetch = 32;  // rays a warp takes from the list per fetch
    int short_stack = -1;     // shared-memory stack entries per thread (-1: default)
    int packets = 1;          // warp-cooperative traversal of the listed rays
    // rays from triangles: list entries (t << 2 | k) are edges of this soup's
    // triangles (the source side's per-join hierarchy)
    const float4* soup = nullptr;
    int64_t bound = -1;       // listed rays at most (-1: the source's edge count)
    int shard_index = 0;      // trace shard shard_index of shard_count of the rays
    int shard_count = 1;
    // rays from a soup: entries[t / entry_group] is the four-wide target
    // node the walks of soup triangle t's edges start at (null: the root)
    const int32_t* entries = nullptr;
    int entry_group = 1;
};

constexpr int kScratchSlots = 40;

// Uniform xy grid over a dataset's object boxes: per cell the objects whose
// box covers the cell in x and y (parity candidates).
struct ColumnGrid {
    int nx = 0, ny = 0;
    const float* bounds = nullptr;   // lo.x, lo.y, hi.x, hi.y (device)
    const int32_t* offsets = nullptr; // nx*ny + 1
    const int32_t* entries = nullptr;
};

constexpr int kSizingScratchSlot = 21;  // 21 and 22: learned sizing (sizing.cu)

struct BvhShape {
    int leaf_size = 1;
    int root_is_leaf = 1;
    int root_leaf_count = 0;
    uint64_t num_nodes = 0;
};

}  // namespace pgpu

// ---- host-side internal objects ------------------------------------------

namespace pgpu {
// Plan of a join captured as a CUDA graph.  The join first runs eagerly
// (mode 1) and records every value it reads back from the device to make a
// host decision (counts that size buffers and launches); the same code then
// runs under stream capture (mode 2), takes those values from the plan
// instead of synchronising, and copies the device's values into pinned
// h_check slots, which a replay compares with the plan.
struct GraphPlan {
    int mode = 0;
    std::vector<int64_t> values;
    std::vector<int> widths;
    size_t cursor = 0;
    std::vector<void*> buffers;        // result buffers of the eager run, reused by the capture
    std::vector<size_t> buffer_bytes;
    size_t buf_cursor = 0;
    int64_t* h_check = nullptr;        // pinned, one slot per value
};
}  // namespace pgpu

struct pierce_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t* d_err = nullptr;
    pgpu::DevCounters* d_counters = nullptr;
    uint32_t* h_err = nullptr;                 // pinned
    pgpu::DevCounters* h_counters = nullptr;   // pinned
    int64_t* h_small = nullptr;                // pinned scratch for scalar readbacks (8 values)
    // grow-only scratch buffers reused across joins
    void* scratch[pgpu::kScratchSlots] = {nullptr};
    size_t scratch_bytes[pgpu::kScratchSlots] = {0};
    // join generation and the generation that last used each slot: a join
    // short of memory frees the slots it has not touched
    uint64_t scratch_gen = 0;
    uint64_t scratch_used[pgpu::kScratchSlots] = {0};
    uint64_t launches = 0;
    int sm_count = 0;
    pgpu::GraphPlan* plan = nullptr;  // set while a join graph is planned or captured
    // dataset uploads: copies and the edge upload kernel run on copy_stream,
    // so the object preparation of the triangles (on stream) overlaps the
    // transfer of the edges
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_tris = nullptr, ev_edges = nullptr;
    int32_t* d_upload_flag = nullptr;  // edges grouped by source object (nonzero) after an upload
    // Dataset arrays come from this stream-ordered pool; freed arrays stay
    // in it up to a quarter of the device's memory, so datasets created and
    // destroyed per query skip the driver's mapping work.
    // pierce_ctx_release_scratch trims it.
    cudaMemPool_t pool = nullptr;
};

struct pierce_dataset {
    pierce_ctx* ctx = nullptr;
    int device = 0;  // ctx->device, kept for release
    uint64_t nv = 0, nt = 0, ne = 0;
    int32_t num_objects = 0;
    float* d_vertices = nullptr;
    uint32_t* d_indices = nullptr;
    int32_t* d_tri_to_object = nullptr;
    float4* d_edges = nullptr;
    int32_t* d_edge_src = nullptr;
    float4* d_soup = nullptr;
    pgpu::Node* d_nodes = nullptr;
    float4* d_first_vertex = nullptr;
    float* d_obj_box = nullptr;
    uint64_t num_nodes = 0;
    int built = 0;
    int root_is_leaf = 0, root_leaf_count = 0;
    int leaf_size = 1;
    double ms_build = 0.0;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    uint64_t device_bytes = 0;
    // partitions (0: none): object -> partition, and the BVH's per-partition roots
    int32_t num_parts = 0;
    int32_t* d_obj_part = nullptr;
    int2* d_part_roots = nullptr;
    // per object (first triangle, triangle count); contiguous = every
    // object's triangles form one index range
    int2* d_obj_range = nullptr;
    int contiguous = 0;
    // boxes of every 32 consecutive triangles and edges (6 floats each)
    float* d_tri_chunk_box = nullptr;
    float* d_edge_chunk_box = nullptr;
    int edges_grouped = 0;  // edge sources non-decreasing (edges grouped by object)
    // hierarchy over the object boxes (with its four-wide copy), which the
    // per-join path culls against: built by the first join that needs it
    // and kept, since it depends only on the objects and their partitions
    void* d_obj_hier = nullptr;
    pgpu::DevDataset obj_hier{};
    int obj_hier_ready = 0;
    // xy column grid over the object boxes (parity candidates when this
    // dataset is the target), kept the same way
    void* d_grid = nullptr;          // bounds, counts and offsets
    void* d_grid_entries = nullptr;  // object ids per cell
    pgpu::ColumnGrid grid{};
    int grid_ready = 0;

    pgpu::DevDataset view() const {
        pgpu::DevDataset v;
        v.soup = d_soup;
        v.nodes = d_nodes;
        v.nodes4 = nullptr;
        v.num_tris = (int64_t)nt;
        v.root_is_leaf = root_is_leaf;
        v.root_leaf_count = root_leaf_count;
        v.edges = d_edges;
        v.edge_src = d_edge_src;
        v.num_edges = (int64_t)ne;
        v.first_vertex = d_first_vertex;
        v.obj_box = d_obj_box;
        v.num_objects = num_objects;
        v.obj_part = d_obj_part;
        v.part_roots = (num_parts && built) ? d_part_roots : nullptr;
        v.verts = d_vertices;
        v.idx = d_indices;
        v.obj_range = contiguous ? d_obj_range : nullptr;
        v.tri_chunk_box = d_tri_chunk_box;
        v.edge_chunk_box = d_edge_chunk_box;
        v.edges_grouped = edges_grouped;
        v.soup_boxes = 0;
        return v;
    }
};

struct pierce_result {
    pierce_pair* d_pairs = nullptr;
    uint64_t count = 0;
    uint64_t capacity = 0;
    uint64_t containment_count = 0;
};

namespace pgpu {
// error reporting (capi.cu)
int set_error(int status, const std::string& msg);
int set_error_cstr(int status, const char* msg);  // never allocates
int check_cuda(cudaError_t e, const char* what);
// grow-only scratch buffer `slot` of at least `bytes`
int scratch(pierce_ctx* ctx, int slot, size_t bytes, void** out);
int device_alloc(void** p, size_t bytes, const char* what);
// dataset arrays: from the context's pool, in order on `stream`; freed by
// dataset_free (after the device is idle)
int dataset_array(pierce_ctx* ctx, void** p, size_t bytes, cudaStream_t stream, const char* what);
void dataset_free(void* p);
// A value the host reads from device memory (4 or 8 bytes, 4 sign-extended):
// synchronous, except while a join graph is captured (then from the plan).
int host_value(pierce_ctx* ctx, const void* dptr, int bytes, int64_t* out, const char* what);
inline bool capturing(const pierce_ctx* ctx) { return ctx->plan && ctx->plan->mode == 2; }
// Device memory of a join result (owned by the join graph while one is planned).
int result_alloc(pierce_ctx* ctx, void** p, size_t bytes);
// allocate a dataset's arrays for ds->nv/nt/ne/num_objects (capi.cu)
int dataset_alloc(pierce_dataset* ds, cudaStream_t stream);
// object data, then the BVH unless tuning->defer_build (capi.cu)
int dataset_finish(pierce_ctx* ctx, pierce_dataset* ds, const pierce_tuning* tuning,
                   cudaEvent_t edges_ready = nullptr, const int32_t* grouped_flag = nullptr);

// sizing.cu: join features into d_out[32] (device), and the network's
// log1p(pairs) prediction for a join (synchronous)
int join_features(pierce_ctx* ctx, const pierce_dataset* A, const pierce_dataset* B, float* d_out);
int learned_log_pairs(pierce_ctx* ctx, const pierce_mlp* mlp, const pierce_dataset* A, const pierce_dataset* B,
                      double* pred);

// lbvh.cu
int build_bvh(pierce_ctx* ctx, pierce_dataset* ds, int leaf_size);
// With obj_part (num_parts > 0) the hierarchy is partitioned: triangles sort
// by (partition of their object, Morton code in the partition's bounds), no
// leaf mixes partitions, and part_roots[p] receives partition p's subtree.
int build_lbvh(pierce_ctx* ctx, const float* verts, const uint32_t* idx, const int32_t* t2o, const uint32_t* list,
               int64_t n, int leaf_size, float4* soup, Node* nodes, BvhShape* shape, float* root_box,
               const int32_t* obj_part = nullptr, int32_t num_parts = 0, int2* part_roots = nullptr);
// Chunk boxes, object boxes, ranges and flags.  With edges_ready (the edge
// upload kernel already wrote the edge chunk boxes and the edge-order flag
// *grouped_flag), the edge-side work waits for ev_edges instead.
// Node4 copy of a binary hierarchy with num_nodes internal nodes
int collapse4(pierce_ctx* ctx, const Node* nodes, int64_t num_nodes, Node4* out);
int prepare_objects(pierce_ctx* ctx, pierce_dataset* ds, cudaEvent_t edges_ready = nullptr,
                    const int32_t* grouped_flag = nullptr);
// hierarchy over groups of G consecutive triangles (G divides 32) of the
// listed 32-triangle chunks; group_scratch holds 96 bytes per group (+ 512).
// With `filter` only the groups whose box meets a leaf of that four-wide
// hierarchy are kept (join.cu k_group_filter); *kept receives their number.
int build_grouped_lbvh(pierce_ctx* ctx, const float* verts, const uint32_t* idx, const int32_t* t2o, int64_t nt,
                       const uint32_t* chunk_list, int64_t n_chunks, int G, void* group_scratch, float4* soup,
                       Node* nodes, BvhShape* shape, const DevDataset* filter = nullptr,
                       unsigned long long* d_count = nullptr, int64_t* kept = nullptr,
                       const int32_t* obj_part = nullptr, int32_t num_parts = 0, int2* part_roots = nullptr);
int launch_group_filter(pierce_ctx* ctx, const float* gbox, int64_t ng, const DevDataset& other,
                        const int32_t* gt2o, const int32_t* obj_part, uint8_t* flags);
// partitioned datasets: *mixed |= some group of a flagged chunk spans two partitions
int launch_group_mixed(pierce_ctx* ctx, const uint8_t* chunk_flags, int64_t n_chunks, const int32_t* t2o,
                       const int32_t* obj_part, int64_t nt, int G, int32_t* mixed);

// sortscan.cu (CUB library calls)
int sort_u32_pairs(pierce_ctx* ctx, uint32_t* keys_in, uint32_t* keys_out, uint32_t* vals_in, uint32_t* vals_out,
                   int64_t n, int end_bit);
int sort_u64_keys(pierce_ctx* ctx, uint64_t* keys_in, uint64_t* keys_out, int64_t n);
int sort_u64_pairs(pierce_ctx* ctx, uint64_t* keys_in, uint64_t* keys_out, uint32_t* vals_in, uint32_t* vals_out,
                   int64_t n, int end_bit);
int exclusive_scan_i32_to_i64(pierce_ctx* ctx, const int32_t* in, int64_t* out, int64_t n);
int exclusive_scan_i32(pierce_ctx* ctx, const int32_t* in, int32_t* out, int64_t n);
int unique_u64(pierce_ctx* ctx, const uint64_t* in, uint64_t* out, int64_t n, int64_t* num_unique);
int select_flagged(pierce_ctx* ctx, const uint8_t* flags, int64_t n, uint32_t* out, unsigned long long* d_count);
}  // namespace pgpu
