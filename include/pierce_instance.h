/*
 * pierce_instance.h — one mesh of an instanced dataset.
 *
 * No counterpart in the reference (its datasets are OBJ files).  The
 * generated workloads are sets of icosphere meshes; a mesh is described by
 * this record and expanded to float32 vertices, triangles and edges either
 * on the host (libpierce_host) or on the device (libpierce_gb300), with the
 * same arithmetic:
 *
 *   u  = unit icosphere template vertex of subdivision `level`
 *   f  = 1 + noise_amp * noise(noise_seed, 1.5 * u + noise_offset)
 *   p  = (axes[0] * u.x * f, axes[1] * u.y * f, axes[2] * u.z * f)
 *   w  = center + rotation * p            (rotation row-major)
 *   vertex = float32(w), each coordinate rounded once
 *
 * where noise() is smooth 3-D value noise in [-1, 1] (hashed lattice values,
 * trilinear interpolation with smoothstep weights).  Everything is IEEE
 * double arithmetic in a fixed order (no fused multiply-add), so host and
 * device expansions are bit-identical.  A sphere of radius r centred at c is
 * axes = (r, r, r), rotation = identity, noise_amp = 0.
 */
#ifndef PIERCE_INSTANCE_H
#define PIERCE_INSTANCE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pierce_mesh_instance {
    double center[3];
    double axes[3];
    double rotation[9];
    double noise_amp;
    double noise_offset[3];
    uint64_t noise_seed;
    int32_t level;          /* icosphere subdivision level, 0..PIERCE_MAX_INSTANCE_LEVEL */
    int32_t group;          /* partition (join of a batch) the mesh belongs to; 0 for a single join */
} pierce_mesh_instance;

#define PIERCE_MAX_INSTANCE_LEVEL 6

#ifdef __cplusplus
}
#endif

#endif /* PIERCE_INSTANCE_H */
