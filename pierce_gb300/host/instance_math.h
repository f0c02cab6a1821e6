// Vertex arithmetic of instanced icosphere meshes, shared by the host
// generators (g++ with -ffp-contract=off) and the device expansion kernels
// (explicit round-to-nearest intrinsics, so nvcc cannot fuse a multiply and
// an add).  Both evaluate the same IEEE double operations in the same order,
// which makes host- and device-expanded datasets bit-identical.
#pragma once

#include <stdint.h>

#include "pierce_instance.h"

#ifdef __CUDACC__
#define PIERCE_HD __host__ __device__ __forceinline__
#else
#define PIERCE_HD inline
#include <cmath>
#endif

namespace pierce {
namespace inst {

PIERCE_HD double dmul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
PIERCE_HD double dadd(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
PIERCE_HD double dsub(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
PIERCE_HD double dfloor(double a) {
#ifdef __CUDA_ARCH__
    return floor(a);
#else
    return std::floor(a);
#endif
}

// splitmix64 finaliser of (h + golden ratio) (Vigna's public-domain mixer).
PIERCE_HD uint64_t mix64(uint64_t h) {
    uint64_t z = h + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// Lattice value in [-1, 1) of integer point (i, j, k).
PIERCE_HD double lattice(uint64_t seed, int64_t i, int64_t j, int64_t k) {
    const uint64_t h = seed ^ ((uint64_t)i * 0x9E3779B97F4A7C15ULL) ^ ((uint64_t)j * 0xC2B2AE3D27D4EB4FULL) ^
                       ((uint64_t)k * 0x165667B19E3779F9ULL);
    return dsub(dmul((double)(mix64(h) >> 11), 2.0 / 9007199254740992.0), 1.0);
}

PIERCE_HD double smoothstep(double t) { return dmul(dmul(t, t), dsub(3.0, dmul(2.0, t))); }

PIERCE_HD double lerp(double a, double b, double t) { return dadd(a, dmul(dsub(b, a), t)); }

// Smooth value noise: trilinear interpolation of the eight surrounding
// lattice values with smoothstep weights.
PIERCE_HD double value_noise(uint64_t seed, double x, double y, double z) {
    const double fx = dfloor(x), fy = dfloor(y), fz = dfloor(z);
    const int64_t i = (int64_t)fx, j = (int64_t)fy, k = (int64_t)fz;
    const double u = smoothstep(dsub(x, fx)), v = smoothstep(dsub(y, fy)), w = smoothstep(dsub(z, fz));
    const double x00 = lerp(lattice(seed, i, j, k), lattice(seed, i + 1, j, k), u);
    const double x10 = lerp(lattice(seed, i, j + 1, k), lattice(seed, i + 1, j + 1, k), u);
    const double x01 = lerp(lattice(seed, i, j, k + 1), lattice(seed, i + 1, j, k + 1), u);
    const double x11 = lerp(lattice(seed, i, j + 1, k + 1), lattice(seed, i + 1, j + 1, k + 1), u);
    return lerp(lerp(x00, x10, v), lerp(x01, x11, v), w);
}

constexpr double kNoiseFrequency = 1.5;

// World position of unit template vertex (ux, uy, uz) of mesh p.
PIERCE_HD void instance_vertex(const pierce_mesh_instance& p, double ux, double uy, double uz, float out[3]) {
    const double n = value_noise(p.noise_seed, dadd(dmul(ux, kNoiseFrequency), p.noise_offset[0]),
                                 dadd(dmul(uy, kNoiseFrequency), p.noise_offset[1]),
                                 dadd(dmul(uz, kNoiseFrequency), p.noise_offset[2]));
    const double f = dadd(1.0, dmul(p.noise_amp, n));
    const double lx = dmul(dmul(p.axes[0], ux), f);
    const double ly = dmul(dmul(p.axes[1], uy), f);
    const double lz = dmul(dmul(p.axes[2], uz), f);
    const double* m = p.rotation;
    out[0] = (float)dadd(p.center[0], dadd(dadd(dmul(m[0], lx), dmul(m[1], ly)), dmul(m[2], lz)));
    out[1] = (float)dadd(p.center[1], dadd(dadd(dmul(m[3], lx), dmul(m[4], ly)), dmul(m[5], lz)));
    out[2] = (float)dadd(p.center[2], dadd(dadd(dmul(m[6], lx), dmul(m[7], ly)), dmul(m[8], lz)));
}

// Sizes of the subdivision-`level` icosphere template.
PIERCE_HD int64_t template_vertices(int level) { return 10ll * (1ll << (2 * level)) + 2; }
PIERCE_HD int64_t template_triangles(int level) { return 20ll << (2 * level); }
PIERCE_HD int64_t template_edges(int level) { return 30ll << (2 * level); }

}  // namespace inst
}  // namespace pierce
