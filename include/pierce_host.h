/*
 * pierce_host.h — host-side C ABI of the Pierce GB300 build: the `.pre`
 * preprocessed-geometry format, unique-edge extraction, grid statistics and
 * the seeded synthetic dataset generators.
 *
 * These entry points replace the reference's header-only format code and its
 * preprocessor helpers (paths relative to the reference project root):
 *   pierce_geom_read_pre      <- RaySpace::IO::readBinaryFile
 *                                pierce/common/include/BinaryIO.h:84-151
 *   pierce_geom_write_pre     <- RaySpace::IO::writeBinaryFile
 *                                pierce/common/include/BinaryIO.h:32-82
 *   pierce_geom_extract_edges <- EdgePreprocessor::extractEdges
 *                                pierce/preprocess/src/EdgePreprocessor.cpp:44-111
 *   pierce_geom_grid_stats    <- generateGridStats
 *                                pierce/preprocess/src/pierce_preprocess.cpp:49-167
 * The generators have no counterpart in the reference (its datasets are
 * external OBJ files); they produce the seeded synthetic workloads.
 *
 * All functions are plain C, take plain pointers and sizes, never call
 * exit(), and report failure through a status code plus
 * pierce_host_last_error().
 */
#ifndef PIERCE_HOST_H
#define PIERCE_HOST_H

#include <stddef.h>
#include <stdint.h>

#include "pierce_instance.h"

#ifdef __cplusplus
extern "C" {
#endif

enum pierce_host_status {
    PIERCE_HOST_OK = 0,
    PIERCE_HOST_ERR_IO = 1,          /* file could not be opened / short read */
    PIERCE_HOST_ERR_MAGIC = 2,       /* header magic is not 0x52334442 */
    PIERCE_HOST_ERR_VERSION = 3,     /* header version is not 4 */
    PIERCE_HOST_ERR_INVALID = 4,     /* invalid argument */
    PIERCE_HOST_ERR_NO_EDGES = 5     /* geometry carries no edge payload */
};

/* Layout of one grid cell record as stored in the file (28 bytes),
 * mirrors SparseGridEntry (pierce/common/include/Geometry.h:15-18) and
 * GridCell (pierce/common/include/GridCell.h:5-10). */
typedef struct pierce_grid_entry {
    int32_t ix, iy, iz;
    uint32_t center_count;
    uint32_t touch_count;
    float avg_size_mean;
    float vol_ratio;
} pierce_grid_entry;

/* Read-only view of a geometry object's arrays (pointers owned by it). */
typedef struct pierce_geom_view {
    const float* vertices;          /* 3 * num_vertices floats (xyz) */
    uint64_t num_vertices;
    const uint32_t* indices;        /* 3 * num_triangles vertex indices */
    uint64_t num_triangles;
    const int32_t* tri_to_object;   /* num_mappings object ids */
    uint64_t num_mappings;
    uint64_t total_triangles;       /* header field totalTriangles */
    const float* edge_starts;       /* 3 * num_edges */
    const float* edge_ends;         /* 3 * num_edges */
    const int32_t* edge_src;        /* num_edges source object ids */
    uint64_t num_edges;
    int32_t has_edges;
    int32_t has_grid;
    float grid_cell_size;
    uint32_t num_grid_cells;
    const pierce_grid_entry* grid_cells;
    int32_t num_objects;            /* max(tri_to_object) + 1, 0 if empty */
} pierce_geom_view;

typedef struct pierce_geom pierce_geom;

const char* pierce_host_last_error(void);

/* Geometry objects. */
int pierce_geom_create(const float* vertices, uint64_t num_vertices,
                       const uint32_t* indices, uint64_t num_triangles,
                       const int32_t* tri_to_object, pierce_geom** out);
void pierce_geom_free(pierce_geom* g);
int pierce_geom_get_view(const pierce_geom* g, pierce_geom_view* out);
int pierce_geom_set_edges(pierce_geom* g, const float* starts, const float* ends,
                          const int32_t* src, uint64_t num_edges);

/* `.pre` v4 I/O. */
int pierce_geom_read_pre(const char* path, pierce_geom** out);
int pierce_geom_write_pre(const pierce_geom* g, const char* path);

/* Unique-edge extraction. order = 0: the reference's map order (keys sorted
 * by quantised start point, end point, object id); order = 1: the same edge
 * set grouped by object (each object's edges in key order). */
int pierce_geom_extract_edges(pierce_geom* g, int order, int num_threads);

/* Grid statistics (per-object AABB, signed volume, sparse cells). */
int pierce_geom_grid_stats(pierce_geom* g, float cell_size);

/* First vertex of every object: vertex x of the object's lowest-index
 * triangle (pierce_containment_main.cpp:336-347).  out: 3*num_objects. */
int pierce_geom_first_vertices(const pierce_geom* g, float* out, int32_t num_objects);

/* ---- seeded synthetic generators ------------------------------------- */

/* Icosphere meshes: radii lognormal(ln_mu, sigma), centres uniform in
 * [lo, hi]^3. level = subdivision level (F = 20*4^level). */
int pierce_gen_icospheres(uint64_t seed, int32_t num_meshes, int32_t level,
                          double ln_mu, double sigma, double lo, double hi,
                          pierce_geom** out);

/* Perturbed ellipsoid pair for intersection/containment stress runs.
 * A: num_a ellipsoids (semi-axes U[axis_lo, axis_hi], random rotation,
 * radial smooth value noise of relative amplitude noise_amp) in [lo,hi]^3.
 * B: num_b meshes of the same kind; frac_inside of them are copies of a
 * random A mesh scaled by inside_scale about its centre, frac_contact of
 * them share exactly coincident vertices or faces with an A mesh. */
int pierce_gen_ellipsoid_pair(uint64_t seed_a, uint64_t seed_b,
                              int32_t num_a, int32_t num_b, int32_t level,
                              double axis_lo, double axis_hi, double noise_amp,
                              double lo, double hi, double frac_inside,
                              double inside_scale, double frac_contact,
                              pierce_geom** out_a, pierce_geom** out_b);

/* Branching tube meshes: random-walk skeleton (step, branch probability
 * per segment), radius U[r_lo, r_hi], n_sides-gon cross sections swept and
 * capped, about target_tris triangles per mesh, starts uniform in [lo,hi]^3.
 * The unique edges are listed per branch as they are built (ring, segment
 * and diagonal edges, cap spokes), the same set unique-edge extraction finds;
 * branches are swept in parallel (OpenMP). */
int pierce_gen_tubes(uint64_t seed, int32_t num_meshes, int64_t target_tris,
                     double step, double branch_prob, double r_lo, double r_hi,
                     int32_t n_sides, double lo, double hi, pierce_geom** out);
/* The first `first_meshes` tubes of pierce_gen_tubes(seed, num_meshes, ...),
 * bit-identical to those meshes of the full dataset (same object ids and
 * coordinates; vertex indices renumbered): samples of a large tube dataset
 * without building all of it. */
int pierce_gen_tubes_head(uint64_t seed, int32_t num_meshes, int32_t first_meshes, int64_t target_tris,
                          double step, double branch_prob, double r_lo, double r_hi,
                          int32_t n_sides, double lo, double hi, pierce_geom** out);

/* Unit icosphere template: counts[0..2] = vertices, triangles, unique edges;
 * any output array may be NULL (query counts first). vertices: 3 doubles each,
 * tris: 3 indices each, edges: 2 indices each (first-seen orientation). */
int pierce_icosphere_template(int32_t level, double* vertices, uint32_t* tris, uint32_t* edges, int64_t* counts);

/* Per-mesh parameters of an instanced dataset (pierce_instance.h).
 * family 0: spheres, radius exp(p0 + p1 * N(0,1)) (p0 = ln mu, p1 = sigma),
 *           drawing the same random stream as pierce_gen_icospheres;
 * family 1: ellipsoids, semi-axes U[p0, p1], uniform random rotation,
 *           radial value noise of relative amplitude noise_amp, drawing the
 *           same stream as side A of pierce_gen_ellipsoid_pair.
 * Centres uniform in [lo, hi]^3; level uniform in [level_lo, level_hi]
 * (no draw when they are equal). */
int pierce_gen_instances(uint64_t seed, int32_t num_meshes, int32_t family, int32_t level_lo, int32_t level_hi,
                         double p0, double p1, double noise_amp, double lo, double hi,
                         pierce_mesh_instance* out);

/* Host expansion of instanced meshes (mesh m = object m); edges are each
 * mesh's unique template edges in template order. */
int pierce_expand_instances(const pierce_mesh_instance* meshes, int32_t num_meshes, pierce_geom** out);

/* Concatenate b onto a (object ids of b shifted by a's object count). */
int pierce_geom_append(pierce_geom* a, const pierce_geom* b);

#ifdef __cplusplus
}
#endif

#endif /* PIERCE_HOST_H */
