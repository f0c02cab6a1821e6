/*
 * pierce_capi.h — C ABI of the GB300 (sm_103a) mesh spatial-join library.
 *
 * The reference has no shared library: its GPU seam is a set of launch
 * parameter structs copied to the device before each optixLaunch plus a few
 * extern "C" helpers.  Each entry point below replaces one of them (paths
 * relative to the reference project root):
 *
 *   pierce_dataset_create / pierce_dataset_build
 *       <- GeometryUploader::upload  pierce/query/src/geometry/GeometryUploader.cpp:12-34
 *          PrecomputedEdgeData::uploadFromGeometry
 *                                    pierce/query/src/geometry/PrecomputedEdgeData.cpp:5-29
 *          OptixAccelerationStructure::build
 *                                    pierce/query/src/optix/OptixAccelerationStructure.cpp:14-68
 *   pierce_launch_edge_rays
 *       <- MeshOverlapEdgesLauncher::launchMesh1ToMesh2 / launchMesh2ToMesh1
 *                                    pierce/query/src/raytracing/MeshOverlapEdgesLauncher.cpp:140-154
 *          (device program __raygen__mesh_overlap_edges,
 *                                    pierce/query/src/cuda/mesh_overlap_edges.cu:105-208;
 *           params MeshOverlapEdgesLaunchParams :12-42)
 *   pierce_launch_parity
 *       <- MeshIntersectionLauncher::launchContainmentMesh1ToMesh2/2To1
 *                                    pierce/query/src/raytracing/MeshIntersectionLauncher.cpp:242-283
 *          MeshContainmentLauncher::launchPointInMesh
 *                                    pierce/query/src/raytracing/MeshContainmentLauncher.cpp:195-213
 *   pierce_parity_tracking
 *       <- PairHitTrackingBuffers / ContainmentTrackingBuffers (--enable-tracking)
 *                                    pierce/query/src/utilities/PairHitTracking.h:31-110,
 *                                    pierce/query/src/utilities/ContainmentTracking.h:22-95
 *   pierce_exclusive_scan
 *       <- exclusive_scan_gpu        pierce/query/src/cuda/scan_utils.h:6-9, scan_utils.cu:11-28
 *   pierce_merge_and_deduplicate_pairs
 *       <- merge_and_deduplicate_pairs_gpu
 *                                    pierce/query/src/cuda/mesh_query_deduplication.h:6-18,
 *                                    mesh_query_deduplication.cu:94-120
 *   pierce_compact_hash_table_pairs
 *       <- compact_hash_table_pairs  pierce/query/src/cuda/mesh_query_deduplication.cu:123-144
 *   pierce_join
 *       <- executeTwoPassQueryEdgesOptimized
 *                                    pierce/query/src/applications/pierce_overlap_two_pass_main.cpp:39-156
 *          executeHashQuery (overlap)
 *                                    pierce/query/src/applications/pierce_overlap_main.cpp:74-187
 *          executeHashQuery (intersection)
 *                                    pierce/query/src/applications/pierce_intersection_main.cpp:78-177
 *          runOnce (containment)     pierce/query/src/applications/pierce_containment_main.cpp:385-550
 *   pierce_estimate_pairs
 *       <- estimateOverlapSelectivity / estimateIntersectionSelectivity
 *                                    pierce/query/src/cuda/estimated_overlap.cu:43-77,
 *                                    estimated_intersection.cu:43-79
 *
 * Conventions: plain C types only; every call returns a pierce_status and
 * never exits the process; a failed call leaves a message for
 * pierce_last_error() (per host thread).  All device work of a context runs
 * on that context's own CUDA stream; one context per host thread.  A dataset
 * keeps indexes built by its first join (the hierarchy and column grid of
 * its object boxes), so two host threads must not start the first joins of
 * one dataset at the same time.
 * Out-of-capacity conditions inside kernels (hash table full, traversal
 * stack overflow, output buffer overflow) come back as status codes.
 * A pair is (object id in dataset A, object id in dataset B), 8 bytes,
 * laid out like MeshQueryResult (pierce/common/include/common.h:34-37).
 */
#ifndef PIERCE_CAPI_H
#define PIERCE_CAPI_H

#include <stddef.h>
#include <stdint.h>

#include "pierce_instance.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pierce_status {
    PIERCE_OK = 0,
    PIERCE_ERR_INVALID_ARGUMENT = 1,
    PIERCE_ERR_CUDA = 2,
    PIERCE_ERR_OUT_OF_MEMORY = 3,
    PIERCE_ERR_NO_DEVICE = 4,
    PIERCE_ERR_HASH_FULL = 5,        /* a hash insert exceeded its probe bound */
    PIERCE_ERR_STACK_OVERFLOW = 6,   /* BVH traversal stack exhausted */
    PIERCE_ERR_OUTPUT_OVERFLOW = 7,  /* result buffer smaller than the pair count */
    PIERCE_ERR_QUEUE_TIMEOUT = 8,    /* bounded wait in a persistent kernel expired */
    PIERCE_ERR_NOT_BUILT = 9         /* dataset has no acceleration structure yet */
} pierce_status;

typedef struct pierce_ctx pierce_ctx;
typedef struct pierce_dataset pierce_dataset;
typedef struct pierce_result pierce_result;
typedef struct pierce_mlp pierce_mlp;

typedef struct pierce_pair {
    int32_t a;  /* object id in dataset A (mesh1) */
    int32_t b;  /* object id in dataset B (mesh2) */
} pierce_pair;

/* Arrays of one preprocessed dataset, as stored in a `.pre` file.  The
 * edges of object o are edges of o's triangles (as pierce_preprocess
 * extracts them): the joins' box culling relies on every edge lying in the
 * boxes of its object's triangles. */
typedef struct pierce_mesh_view {
    const float* vertices;        /* 3 * num_vertices (xyz) */
    uint64_t num_vertices;
    const uint32_t* indices;      /* 3 * num_triangles */
    uint64_t num_triangles;
    const int32_t* tri_to_object; /* num_triangles */
    const float* edge_starts;     /* 3 * num_edges */
    const float* edge_ends;       /* 3 * num_edges */
    const int32_t* edge_src;      /* num_edges source object ids */
    uint64_t num_edges;
    int32_t num_objects;          /* max object id + 1; < 0: computed by the library */
    /* Optional, for meshes stored object by object (as `.pre` files are):
       object o holds triangles [object_offsets[o], object_offsets[o + 1]),
       num_objects + 1 non-decreasing entries from 0 to num_triangles, always
       in host memory.  When given (num_objects >= 0), tri_to_object may be
       NULL and is not read: the library writes the per-triangle object ids
       on the device, so the upload moves 8 bytes per object instead of 4 per
       triangle. */
    const int64_t* object_offsets;
} pierce_mesh_view;

enum pierce_memory { PIERCE_HOST_MEMORY = 0, PIERCE_DEVICE_MEMORY = 1 };

typedef enum pierce_predicate {
    PIERCE_OVERLAP = 0,       /* surfaces meet: edge rays both ways */
    PIERCE_INTERSECTION = 1,  /* overlap U first-vertex parity both ways */
    PIERCE_CONTAINMENT = 2    /* B's first vertex inside A by parity, minus overlap */
} pierce_predicate;

typedef enum pierce_direction {
    PIERCE_BOTH = 0,
    PIERCE_MESH1_TO_MESH2 = 1,
    PIERCE_MESH2_TO_MESH1 = 2
} pierce_direction;

typedef enum pierce_sizing {
    PIERCE_SIZING_TWO_PASS = 0,   /* count, scan, write, sort + unique */
    PIERCE_SIZING_HASH = 1,       /* hash set sized from expected_pairs */
    PIERCE_SIZING_FIXED = 2,      /* hash set of hash_table_slots slots */
    PIERCE_SIZING_LEARNED = 3     /* hash set sized by sizing_model's prediction x output_safety;
                                     two-pass rerun when the pairs do not fit */
} pierce_sizing;

typedef enum pierce_precision {
    PIERCE_EXACT = 0,   /* FP32 filter, FP64 then exact expansion fallback */
    PIERCE_FP32 = 1     /* plain float32 Moller-Trumbore, no fallback */
} pierce_precision;

typedef struct pierce_tuning {
    int32_t leaf_size;        /* max triangles per BVH leaf (1..8) */
    int32_t block_size;       /* threads per block for traversal kernels */
    int32_t sort_rays;        /* 1: trace edge rays in Morton order of their midpoints */
    int32_t cull_objects;     /* 1: skip source objects whose box meets no target object */
    int32_t defer_build;      /* 1: pierce_dataset_create uploads only; call pierce_dataset_build */
    int32_t skip_edges;       /* 1: pierce_dataset_create neither reads nor uploads the view's edge arrays
                                 (joins then take their rays from the triangles: edge_source) */
} pierce_tuning;

/* Where a join's edge rays come from (pierce_join_opts.edge_source). */
enum pierce_edge_source {
    PIERCE_EDGES_AUTO = 0,       /* per side: the kept triangles' edges where the join builds grouped
                                    per-join hierarchies and the side keeps fewer than half of its
                                    triangles, else the dataset's edges (triangles when it has none) */
    PIERCE_EDGES_DATASET = 1,    /* the dataset's edge list (the `.pre` edges) */
    PIERCE_EDGES_TRIANGLES = 2   /* the edges of the triangles kept for the join's per-join hierarchies, each
                                    segment of a leaf group once (needs active_bvh) */
};

typedef struct pierce_join_opts {
    int32_t predicate;            /* pierce_predicate */
    int32_t direction;            /* pierce_direction */
    int32_t sizing;               /* pierce_sizing */
    int32_t precision;            /* pierce_precision */
    uint64_t expected_pairs;      /* HASH sizing input (0: default table) */
    uint64_t hash_table_slots;    /* FIXED sizing */
    double hash_load_factor;      /* (0,1], default 0.5 */
    double output_safety;         /* result capacity = expected * safety (>= 1) */
    int32_t include_overlap_pairs;/* containment: also report overlap pairs */
    int32_t max_retries;          /* table/output enlargements before failing */
    int32_t cull_objects;         /* 1 (default): skip edges of source objects whose box meets no target triangle box */
    int32_t defer_exact;          /* 1 (default): queue FP32-undecided tests for a separate exact pass */
    int32_t active_bvh;           /* 1 (default): build per-join BVHs over the triangles of objects whose box
                                     meets an object box of the other side (datasets need no BVH of their own) */
    const pierce_mlp* sizing_model; /* LEARNED sizing: trained network (pierce_mlp_create) */
    /* tuning (0: default); pierce_autotune_join picks them */
    int32_t leaf_size;            /* leaf size of the per-join hierarchies (0: the datasets' when above 1, else 4) */
    int32_t rays_per_warp;        /* rays a warp takes per fetch from the ray queue (multiple of 32; 0: 32) */
    int32_t stack_depth;          /* traversal stack entries in shared memory per thread (1..32; 0: 8 for culled
                                     rays, 32 otherwise) */
    int32_t traversal;            /* culled rays: 0 one ray per thread over four-wide copies of the per-join
                                     hierarchies, 1 a warp traverses its 32 rays together, 2 one ray per thread
                                     over the binary nodes */
    int32_t edge_source;          /* pierce_edge_source.  Exact predicates give the same pairs from either
                                     source when the dataset's edges are its triangles' edges (as
                                     pierce_preprocess extracts them): a segment's hits do not depend on
                                     its orientation */
    /* Shard shard_index of shard_count (0 or 1: the whole join), for one
     * process per GPU: each edge ray belongs to one shard by a hash of its
     * segment's endpoints (rays from triangles) or by its range of edge
     * indices (the dataset's edges), and the parity rays by ranges of source
     * objects; the union of the shards' pairs is the join's pair set
     * (overlap, intersection).  Containment is split by
     * B object (each shard's pairs are those of its B objects; needs
     * active_bvh, both datasets' objects stored contiguously and no
     * include_overlap_pairs).  Every shard builds the same per-join
     * hierarchies. */
    int32_t shard_index;
    int32_t shard_count;
    int32_t reserved;
} pierce_join_opts;

typedef struct pierce_stats {
    double ms_total;              /* GPU time of the whole join (CUDA events) */
    double ms_edge_rays[2];       /* A->B, B->A edge-ray kernels (all passes) */
    double ms_parity[2];          /* A->B, B->A parity kernels */
    double ms_dedup;              /* scan, sort/unique or compaction */
    uint64_t rays;                /* edge rays traced (per pass) */
    uint64_t node_visits;         /* BVH nodes fetched */
    uint64_t tri_tests;           /* ray-triangle tests */
    uint64_t raw_hits;            /* pair emissions before deduplication */
    uint64_t fp32_ambiguous;      /* predicates the FP32 filter could not decide */
    uint64_t fp64_ambiguous;      /* ... and the FP64 filter could not decide */
    uint64_t parity_rays;
    uint64_t hash_slots;          /* hash table slots used by the join */
    uint64_t result_capacity;     /* pairs the result buffer could hold */
    uint64_t num_pairs;           /* pairs in the result */
    uint64_t overlap_pairs;       /* containment: overlap pairs found */
    uint64_t containment_pairs;   /* containment: strict containment pairs */
    int32_t retries;              /* enlargements performed */
    int32_t launches;             /* kernels launched by the join */
    double ms_count_pass[2];      /* two-pass: pass-1 (count) share of ms_edge_rays */
    uint64_t raw_pairs[2];        /* raw pair emissions A->B, B->A (two-pass pass 1) */
    uint64_t hash_accesses;       /* hash slot inspections */
    uint64_t hash_contentions;    /* inspections past the first slot of a probe */
    double ms_build;              /* per-join BVH builds (active_bvh) */
    uint64_t active_triangles[2]; /* triangles in the per-join BVHs of A and B */
    double predicted_pairs;       /* LEARNED sizing: the network's pair-count prediction */
    double ms_sizing;             /* LEARNED sizing: features + inference */
    int32_t sizing_overflow;      /* LEARNED sizing: 1 when the pairs exceeded the predicted capacity
                                     and the join was rerun two-pass */
    int32_t containment_by_pairs; /* containment: 1 when the odd-parity candidate pairs were tested directly
                                     (no per-join hierarchies were built) */
} pierce_stats;

typedef struct pierce_dataset_info {
    uint64_t num_vertices, num_triangles, num_edges;
    int32_t num_objects;
    int32_t built;
    uint64_t num_nodes;
    uint64_t device_bytes;
    double ms_build;              /* GPU time of the last build */
    float bounds_lo[3], bounds_hi[3];
    int32_t num_parts;            /* partitions (0: not partitioned) */
    int32_t objects_contiguous;   /* 1: every object's triangles form one index range */
    int32_t reserved;
} pierce_dataset_info;

/* ---- context ------------------------------------------------------------ */
const char* pierce_last_error(void);
const char* pierce_status_string(int status);
int pierce_ctx_create(int device, pierce_ctx** out);
void pierce_ctx_destroy(pierce_ctx* ctx);
int pierce_ctx_synchronize(pierce_ctx* ctx);
/* The context's CUDA stream (cudaStream_t), for callers that time or order
 * their own work against the library's. */
void* pierce_ctx_stream(pierce_ctx* ctx);
void pierce_default_tuning(pierce_tuning* t);
void pierce_default_join_opts(pierce_join_opts* o);
/* Kernels launched by this context since its creation. */
uint64_t pierce_ctx_kernel_launches(const pierce_ctx* ctx);
/* Free the context's join scratch memory (kept and reused across joins
 * otherwise; the next join allocates it again). */
int pierce_ctx_release_scratch(pierce_ctx* ctx);
/* Free and total memory of the context's device (cudaMemGetInfo). */
int pierce_device_memory(pierce_ctx* ctx, uint64_t* free_bytes, uint64_t* total_bytes);

/* ---- datasets ----------------------------------------------------------- */
/* Copy a dataset to the device (from host or device memory) and build its
 * bounding-volume hierarchy (tuning may be NULL for defaults). */
int pierce_dataset_create(pierce_ctx* ctx, const pierce_mesh_view* view, int memory,
                          const pierce_tuning* tuning, pierce_dataset** out);
/* Generated datasets (no counterpart in the reference, whose datasets are
 * OBJ files): expand num_meshes instanced icosphere meshes (host array,
 * pierce_instance.h) directly into device memory, mesh m = object m, edges in
 * template order; bit-identical to the host's pierce_expand_instances. */
int pierce_dataset_create_instanced(pierce_ctx* ctx, const pierce_mesh_instance* meshes, int32_t num_meshes,
                                    const pierce_tuning* tuning, pierce_dataset** out);
/* Batches of independent joins: partition a dataset's objects (host array
 * obj_part[num_objects], ids in [0, num_parts)).  Joining two datasets with
 * the same partition count joins partition p of A with partition p of B
 * only, for every p, in the same launches (one hierarchy per dataset with a
 * subtree per partition).  num_parts = 0 removes the partitioning.  A built
 * dataset is rebuilt.  No counterpart in the reference (one join per run). */
int pierce_dataset_set_partitions(pierce_ctx* ctx, pierce_dataset* ds, const int32_t* obj_part, int32_t num_parts);
/* Copy a dataset's arrays back to host memory (sizes from
 * pierce_dataset_info_get; any pointer may be NULL).  Synchronous. */
int pierce_dataset_download(pierce_ctx* ctx, const pierce_dataset* ds, float* vertices, uint32_t* indices,
                            int32_t* tri_to_object, float* edge_starts, float* edge_ends, int32_t* edge_src);
/* Rebuild the hierarchy (e.g. with another leaf size). */
int pierce_dataset_build(pierce_ctx* ctx, pierce_dataset* ds, const pierce_tuning* tuning);
int pierce_dataset_info_get(const pierce_dataset* ds, pierce_dataset_info* out);
/* Release a dataset (also valid after its context was destroyed). */
void pierce_dataset_destroy(pierce_dataset* ds);

/* ---- joins -------------------------------------------------------------- */
/* Full join of A (mesh1) and B (mesh2); the result holds the unique pairs
 * sorted by (a, b), resident on the device. stats may be NULL. */
int pierce_join(pierce_ctx* ctx, pierce_dataset* a, pierce_dataset* b, const pierce_join_opts* opts,
                pierce_result** out, pierce_stats* stats);
int pierce_result_count(const pierce_result* r, uint64_t* count);
/* Device pointer to the result's pierce_pair array. */
const pierce_pair* pierce_result_device_pairs(const pierce_result* r);
/* Copy up to `capacity` pairs to host memory (synchronous). */
int pierce_result_copy(pierce_ctx* ctx, const pierce_result* r, pierce_pair* host_out, uint64_t capacity);
/* Containment with include_overlap_pairs: number of leading result entries
 * that are strict containment pairs (the rest are overlap pairs). */
int pierce_result_containment_count(const pierce_result* r, uint64_t* count);
void pierce_result_destroy(pierce_result* r);

/* ---- autotuning ------------------------------------------------------------ */
/* No counterpart in the reference.  Times the join (a, b) with `base`
 * options over a grid of tuning values, one parameter at a time (leaf size
 * of the per-join hierarchies {1, 2, 4, 8} when base->active_bvh, rays per
 * warp {32, 64, 128}, stack depth {8, 16, 32}, hash load factor
 * {0.25, 0.5, 0.75} when the sizing uses a hash set, traversal {one ray per
 * thread over four-wide nodes, warp packets, one ray per thread over binary
 * nodes}, and the rays' source {as in base, the datasets' edges} when both
 * datasets hold edges), each trial the best
 * of `repeats` timed runs after one untimed run.  *best receives the
 * fastest values; trials[0 .. *num_trials) every trial (max_trials slots,
 * may be NULL). */
typedef struct pierce_tuned {
    int32_t leaf_size;
    int32_t rays_per_warp;
    int32_t stack_depth;
    int32_t traversal;
    int32_t edge_source;          /* pierce_edge_source */
    int32_t reserved;
    double hash_load_factor;
    double ms;                    /* best GPU time of the join with these values */
} pierce_tuned;
int pierce_autotune_join(pierce_ctx* ctx, pierce_dataset* a, pierce_dataset* b, const pierce_join_opts* base,
                         int32_t repeats, pierce_tuned* best, pierce_tuned* trials, int32_t max_trials,
                         int32_t* num_trials);

/* ---- joins captured as CUDA graphs -------------------------------------- */
/* No counterpart in the reference (whose launches are synchronous, one
 * optixLaunch per pass).  pierce_join_graph_create runs the join once
 * (stats of that run in *stats), recording every value the host reads back
 * to size buffers and launches, then captures the same join as one CUDA
 * graph that uses those values and its own scratch memory.  Each
 * pierce_join_graph_launch replays the whole join with one cudaGraphLaunch
 * and one synchronisation; the replay checks that the device produced the
 * recorded values and fails with PIERCE_ERR_OUTPUT_OVERFLOW otherwise (the
 * inputs changed: create a new graph).  The datasets and the sizing model
 * must stay alive and unchanged while the graph exists, and the context
 * must outlive it.  The graph takes over the context's scratch memory and
 * returns it when destroyed.  The pairs of the last replay (sorted by
 * (a, b)) stay in graph-owned device memory. */
typedef struct pierce_join_graph pierce_join_graph;
int pierce_join_graph_create(pierce_ctx* ctx, pierce_dataset* a, pierce_dataset* b, const pierce_join_opts* opts,
                             pierce_join_graph** out, pierce_stats* stats);
int pierce_join_graph_launch(pierce_ctx* ctx, pierce_join_graph* g, pierce_stats* stats);
int pierce_join_graph_pairs(const pierce_join_graph* g, const pierce_pair** d_pairs, uint64_t* count);
int pierce_join_graph_copy(pierce_ctx* ctx, const pierce_join_graph* g, pierce_pair* host_out, uint64_t capacity);
void pierce_join_graph_destroy(pierce_join_graph* g);

/* ---- launch-level entry points (the reference's launcher seam) ---------- */
enum pierce_ray_mode { PIERCE_RAYS_COUNT = 0, PIERCE_RAYS_WRITE = 1, PIERCE_RAYS_HASH = 2 };

/* Edge rays of `src` against `tgt`'s triangles.  COUNT writes d_counts[e]
 * (hits per edge after per-edge de-duplication of target objects); WRITE
 * stores pair keys ((a << 32) | b, uint64) at d_keys[d_offsets[e] ...];
 * HASH inserts the keys into the open-addressing set d_table of
 * table_slots slots (a power of two; empty slot = all ones).  swap != 0
 * stores (target, source) instead of (source, target). */
int pierce_launch_edge_rays(pierce_ctx* ctx, const pierce_dataset* src, const pierce_dataset* tgt, int mode,
                            int precision, int swap, int32_t* d_counts, const int64_t* d_offsets,
                            uint64_t* d_keys, uint64_t* d_table, uint64_t table_slots, pierce_stats* stats);
/* First-vertex +Z parity rays of `src` objects against `tgt`: toggles the
 * parity of key (src, tgt) (or (tgt, src) when swap) in the set d_table /
 * d_parity (table_slots slots). */
int pierce_launch_parity(pierce_ctx* ctx, const pierce_dataset* src, const pierce_dataset* tgt, int precision,
                         int swap, uint64_t* d_table, uint32_t* d_parity, uint64_t table_slots,
                         pierce_stats* stats);
/* Diagnostics of the parity rays (pierce_intersection --enable-tracking):
 * the +Z ray from the first vertex of every object s of `src` against the
 * objects of `tgt`, whose triangles must be stored object by object
 * (objects_contiguous in pierce_dataset_info).  Host arrays, n = src's
 * object count, any of them may be NULL:
 *   target_ids[n * max_targets], target_hits[n * max_targets]: from
 *     s * max_targets on, the target objects s's ray crosses an odd number
 *     of times (s inside them by parity) and their crossing counts;
 *     unused slots hold -1 and 0;
 *   targets_crossed[n]: the target objects s's ray crosses at all;
 *   overflows[n]: odd targets that found no slot.
 * Objects without triangles trace no ray (all zero).  Partitioned datasets:
 * targets of the source's partition only.  Synchronous.  Counterpart of
 * the reference's pair-hit and containment tracking buffers
 * (pierce/query/src/utilities/PairHitTracking.h:31-110,
 * ContainmentTracking.h:22-95), filled by __raygen__mesh_containment_anyhit
 * (pierce/query/src/cuda/mesh_intersection_anyhit.cu:108-146). */
int pierce_parity_tracking(pierce_ctx* ctx, const pierce_dataset* src, const pierce_dataset* tgt, int32_t max_targets,
                           int32_t* target_ids, uint32_t* target_hits, uint32_t* targets_crossed,
                           uint32_t* overflows);

/* ---- helpers replacing the reference's extern "C" device helpers -------- */
/* Exclusive scan of n int32 counts into int64 offsets; *total = sum. */
int pierce_exclusive_scan(pierce_ctx* ctx, const int32_t* d_counts, int64_t* d_offsets, int64_t n,
                          int64_t* total);
/* Sort + unique of the concatenation of two device pair arrays written to
 * d_out (which may alias d_pairs1); pairs end sorted by (a, b). */
int pierce_merge_and_deduplicate_pairs(pierce_ctx* ctx, const pierce_pair* d_pairs1, int64_t n1,
                                       const pierce_pair* d_pairs2, int64_t n2, pierce_pair* d_out,
                                       int64_t* num_unique);
/* Compact the occupied slots of a pair-key hash set into d_out (at most
 * max_output pairs, unsorted); *count = number of occupied slots, which may
 * exceed max_output (then PIERCE_ERR_OUTPUT_OVERFLOW is returned). */
int pierce_compact_hash_table_pairs(pierce_ctx* ctx, const uint64_t* d_table, uint64_t table_slots,
                                    pierce_pair* d_out, uint64_t max_output, uint64_t* count);

/* ---- de-duplication without allocation ---------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory where they need unique pairs: code that runs between stream-ordered
 * steps and must not let cudaMalloc/cudaFree synchronise the device, and
 * plug-ins whose host application owns the memory budget.  The caller passes
 * the input pairs, an output array of at least n pairs and a device word for
 * the unique count; the scratch is a hash set in a fixed device array of
 * PIERCE_NOALLOC_TABLE_SLOTS 64-bit slots (32 MiB) that every GPU loading
 * this library holds until the process exits.  Inputs larger than
 * PIERCE_NOALLOC_MAX_PAIRS pairs are rejected with
 * PIERCE_ERR_INVALID_ARGUMENT.  The call enqueues its work on `stream` (a
 * cudaStream_t of the current device) and returns without waiting; the
 * unique pairs land in d_out[0 .. *d_num_unique) in no particular order.
 * Every call looks up the array's device address (cudaGetSymbolAddress,
 * which allocates nothing); the first call on a device also clears the
 * array (it starts zeroed), so make that first call before any stream
 * capture.  Each call leaves the table empty for the next one.  The pair
 * (-1, -1) is accepted like any other.  All calls share the one array, so
 * calls whose work overlaps on the GPU race: order them on one stream. */
#define PIERCE_NOALLOC_TABLE_SLOTS (1u << 22)
#define PIERCE_NOALLOC_MAX_PAIRS (1u << 21)
int pierce_deduplicate_pairs_noalloc(const pierce_pair* d_pairs, int64_t n, pierce_pair* d_out,
                                     uint64_t* d_num_unique, void* stream);

/* ---- output sizing ------------------------------------------------------ */
/* Grid selectivity estimate (GridCell statistics of both datasets); the
 * cells arrays are host memory of 28-byte records {int3 index; u32 center;
 * u32 touch; f32 avg_size; f32 vol_ratio}. Returns the raw sum over matched
 * cells in *raw and the alpha-corrected estimate in *estimate. */
int pierce_estimate_pairs(pierce_ctx* ctx, const void* cells_a, uint32_t num_a, const void* cells_b,
                          uint32_t num_b, float cell_size, float epsilon, float gamma, int alpha_correction,
                          double* raw, int64_t* estimate, int32_t* matched_cells);

/* ---- learned output sizing ---------------------------------------------- */
/* No counterpart in the reference (whose sizing is the grid estimate above).
 * A 32-64-64-1 FP32 network (ReLU) predicts log(1 + unique pairs) of a join
 * from 32 summary features of its datasets (pierce_join_features).  Weights
 * are row-major: W1[64][32], b1[64], W2[64][64], b2[64], W3[64], b3; inputs
 * are standardised with x_mean / x_scale and the output is de-standardised
 * as o * y_std + y_mean.  Training (Adam, mean squared error on the
 * standardised log counts) and inference run on the device. */
#define PIERCE_MLP_INPUTS 32
#define PIERCE_MLP_HIDDEN 64
#define PIERCE_MLP_PARAMS (PIERCE_MLP_HIDDEN * PIERCE_MLP_INPUTS + PIERCE_MLP_HIDDEN + \
                           PIERCE_MLP_HIDDEN * PIERCE_MLP_HIDDEN + PIERCE_MLP_HIDDEN + PIERCE_MLP_HIDDEN + 1)

typedef struct pierce_mlp_params {
    float weights[PIERCE_MLP_PARAMS];
    float x_mean[PIERCE_MLP_INPUTS];
    float x_scale[PIERCE_MLP_INPUTS];
    float y_mean;
    float y_std;
} pierce_mlp_params;

typedef struct pierce_mlp_train_opts {
    uint64_t seed;                /* sample order */
    int32_t epochs;
    int32_t fit_normalization;    /* 1: set x_mean/x_scale/y_mean/y_std from the training data first */
    float lr, beta1, beta2, eps;  /* Adam */
} pierce_mlp_train_opts;

void pierce_default_mlp_train_opts(pierce_mlp_train_opts* o);
/* Deterministic He-uniform initial weights, zero biases, identity scaling. */
int pierce_mlp_init_params(pierce_mlp_params* p, uint64_t seed);
int pierce_mlp_create(pierce_ctx* ctx, const pierce_mlp_params* init, pierce_mlp** out);
void pierce_mlp_destroy(pierce_mlp* m);
int pierce_mlp_get(pierce_ctx* ctx, const pierce_mlp* m, pierce_mlp_params* out);
/* Train on n samples (host arrays X[n][32], y[n] = log1p(pairs)); the
 * per-epoch mean loss goes to loss_per_epoch (host, epochs floats; may be NULL). */
int pierce_mlp_train(pierce_ctx* ctx, pierce_mlp* m, const float* X, const float* y, int32_t n,
                     const pierce_mlp_train_opts* opts, float* loss_per_epoch);
/* Gradient of the mean squared error over the n samples (host grad[PIERCE_MLP_PARAMS]). */
int pierce_mlp_gradient(pierce_ctx* ctx, const pierce_mlp* m, const float* X, const float* y, int32_t n,
                        float* grad, float* loss);
/* Predicted log1p(pairs) for n feature rows (host arrays). */
int pierce_mlp_predict(pierce_ctx* ctx, const pierce_mlp* m, const float* X, int32_t n, float* out);
/* The 32 features of the join (a, b) into host out[32]. */
int pierce_join_features(pierce_ctx* ctx, const pierce_dataset* a, const pierce_dataset* b, float* out);

#ifdef __cplusplus
}
#endif

#endif /* PIERCE_CAPI_H */
