// Geometric predicates of the join kernels.
//
// Every decision is the sign of a polynomial in the float32 input
// coordinates.  Evaluation is staged:
//   1. float32 with a forward error bound: the value is trusted when its
//      magnitude exceeds 12 * 2^-24 times the permanent (the same polynomial
//      evaluated on absolute values).  Each monomial of a 3x3 determinant of
//      coordinate differences passes through at most 8 roundings (3 input
//      differences, 2 products, 1 subtraction, 2 additions), so the rounding
//      error is below 8.01 * eps * permanent; 12 leaves margin for the
//      rounding of the permanent itself.  Fused multiply-adds only remove
//      roundings and keep the bound valid.
//   2. float64 with the analogous bound (eps = 2^-53);
//   3. exact evaluation with floating-point expansions (Shewchuk 1997,
//      "Adaptive Precision Floating-Point Arithmetic and Fast Robust
//      Geometric Predicates": Two-Sum, Two-Product, Fast-Expansion-Sum and
//      Scale-Expansion with zero elimination), restated here.  Differences
//      of the float inputs are formed exactly as two-term expansions.
// Stages 2-3 run only for the (rare) undecided predicates and live in
// non-inlined functions so that their local arrays do not burden the hot
// traversal loop.
//
// The predicates are:
//   orient3d(a,b,c,d) = sign det[b-a, c-a, d-a]
//   orient2d(a,b,c; i,j) = sign ((b_i-a_i)(c_j-a_j) - (b_j-a_j)(c_i-a_i))
// and the two tests built from them:
//   seg_tri:     closed segment pq meets closed triangle abc (zero-area
//                triangles never meet anything);
//   zray_cross:  the +Z ray from p crosses triangle abc, with p perturbed
//                by (eps, eps^2) in (x, y) so it never lies on a projected
//                edge, vertical triangles never crossed, and the triangle
//                counted only if strictly above p.
// The plain float32 Moller-Trumbore test (no fallback) is also here; its
// operation order is fixed with round-to-nearest intrinsics so that a CPU
// restatement compiled without contraction reproduces it bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pgpu {

struct PredCounters {
    uint32_t fp32_ambiguous;
    uint32_t fp64_ambiguous;
};

// ---------------------------------------------------------------- expansions
__device__ __forceinline__ void two_sum(double a, double b, double& x, double& y) {
    x = __dadd_rn(a, b);
    double bv = __dsub_rn(x, a);
    double av = __dsub_rn(x, bv);
    y = __dadd_rn(__dsub_rn(a, av), __dsub_rn(b, bv));
}
__device__ __forceinline__ void fast_two_sum(double a, double b, double& x, double& y) {
    // requires |a| >= |b|
    x = __dadd_rn(a, b);
    y = __dsub_rn(b, __dsub_rn(x, a));
}
__device__ __forceinline__ void two_diff(double a, double b, double& x, double& y) {
    x = __dsub_rn(a, b);
    double bv = __dsub_rn(a, x);
    double av = __dadd_rn(x, bv);
    y = __dadd_rn(__dsub_rn(a, av), __dsub_rn(bv, b));
}
__device__ __forceinline__ void two_prod(double a, double b, double& x, double& y) {
    x = __dmul_rn(a, b);
    y = __fma_rn(a, b, -x);
}

// h = e + f (both non-overlapping, increasing magnitude); returns |h|.
__device__ __noinline__ int exp_sum(int elen, const double* e, int flen, const double* f, double* h) {
    if (elen == 0) {
        for (int i = 0; i < flen; ++i) h[i] = f[i];
        return flen;
    }
    if (flen == 0) {
        for (int i = 0; i < elen; ++i) h[i] = e[i];
        return elen;
    }
    int i = 0, j = 0, k = 0;
    auto next = [&]() -> double {
        if (j >= flen || (i < elen && fabs(e[i]) < fabs(f[j]))) return e[i++];
        return f[j++];
    };
    double Q = next();
    double g = next();
    double hh;
    fast_two_sum(g, Q, Q, hh);
    if (hh != 0.0) h[k++] = hh;
    while (i < elen || j < flen) {
        g = next();
        two_sum(Q, g, Q, hh);
        if (hh != 0.0) h[k++] = hh;
    }
    if (Q != 0.0 || k == 0) h[k++] = Q;
    return k;
}

// h = e * b; returns |h|.
__device__ __noinline__ int exp_scale(int elen, const double* e, double b, double* h) {
    if (elen == 0 || b == 0.0) {
        h[0] = 0.0;
        return 1;
    }
    int k = 0;
    double Q, hh;
    two_prod(e[0], b, Q, hh);
    if (hh != 0.0) h[k++] = hh;
    for (int i = 1; i < elen; ++i) {
        double p1, p0, s;
        two_prod(e[i], b, p1, p0);
        two_sum(Q, p0, s, hh);
        if (hh != 0.0) h[k++] = hh;
        fast_two_sum(p1, s, Q, hh);
        if (hh != 0.0) h[k++] = hh;
    }
    if (Q != 0.0 || k == 0) h[k++] = Q;
    return k;
}

// h = e * f for short expansions (|e|, |f| <= 16); returns |h|.
__device__ __noinline__ int exp_mul(int elen, const double* e, int flen, const double* f, double* h) {
    double acc[64], tmp[32], sum[64];
    int alen = 0;
    for (int k = 0; k < flen; ++k) {
        int tlen = exp_scale(elen, e, f[k], tmp);
        int slen = exp_sum(alen, acc, tlen, tmp, sum);
        for (int i = 0; i < slen; ++i) acc[i] = sum[i];
        alen = slen;
    }
    for (int i = 0; i < alen; ++i) h[i] = acc[i];
    return alen;
}

__device__ __forceinline__ int exp_negate(int n, double* e) {
    for (int i = 0; i < n; ++i) e[i] = -e[i];
    return n;
}

__device__ __forceinline__ int exp_sign(int n, const double* e) {
    double top = e[n - 1];
    return top > 0.0 ? 1 : (top < 0.0 ? -1 : 0);
}

// exact difference b - a of two floats as an expansion (1 or 2 terms)
__device__ __forceinline__ int exp_diff(float b, float a, double* h) {
    double x, y;
    two_diff((double)b, (double)a, x, y);
    if (y != 0.0) {
        h[0] = y;
        h[1] = x;
        return 2;
    }
    h[0] = x;
    return 1;
}

// exact sign of det[u, v, w] with u, v, w given as coordinate differences
// (expansions of length <= 2 each).
__device__ __noinline__ int exact_det3(const double* u, const int* ul, const double* v, const int* vl,
                                       const double* w, const int* wl) {
    // cofactor c_i = v_j w_k - v_k w_j; det = sum u_i c_i
    double p1[8], p2[8], c[16], t[64], acc[192], acc2[192];
    int alen = 0;
    for (int i = 0; i < 3; ++i) {
        const int j = (i + 1) % 3, k = (i + 2) % 3;
        int l1 = exp_mul(vl[j], v + 2 * j, wl[k], w + 2 * k, p1);
        int l2 = exp_mul(vl[k], v + 2 * k, wl[j], w + 2 * j, p2);
        exp_negate(l2, p2);
        int lc = exp_sum(l1, p1, l2, p2, c);
        int lt = exp_mul(ul[i], u + 2 * i, lc, c, t);
        int ls = exp_sum(alen, acc, lt, t, acc2);
        for (int q = 0; q < ls; ++q) acc[q] = acc2[q];
        alen = ls;
    }
    return alen ? exp_sign(alen, acc) : 0;
}

__device__ __noinline__ int orient3d_exact(float3 a, float3 b, float3 c, float3 d) {
    double u[6], v[6], w[6];
    int ul[3], vl[3], wl[3];
    const float A[3] = {a.x, a.y, a.z}, B[3] = {b.x, b.y, b.z}, C[3] = {c.x, c.y, c.z}, D[3] = {d.x, d.y, d.z};
    for (int i = 0; i < 3; ++i) {
        ul[i] = exp_diff(B[i], A[i], u + 2 * i);
        vl[i] = exp_diff(C[i], A[i], v + 2 * i);
        wl[i] = exp_diff(D[i], A[i], w + 2 * i);
    }
    return exact_det3(u, ul, v, vl, w, wl);
}

__device__ __forceinline__ float fcomp(float3 p, int k) { return k == 0 ? p.x : (k == 1 ? p.y : p.z); }

__device__ __noinline__ int orient2d_exact(float3 a, float3 b, float3 c, int i, int j) {
    double u0[2], u1[2], v0[2], v1[2], p1[8], p2[8], r[16];
    int l_u0 = exp_diff(fcomp(b, i), fcomp(a, i), u0);
    int l_u1 = exp_diff(fcomp(b, j), fcomp(a, j), u1);
    int l_v0 = exp_diff(fcomp(c, i), fcomp(a, i), v0);
    int l_v1 = exp_diff(fcomp(c, j), fcomp(a, j), v1);
    int l1 = exp_mul(l_u0, u0, l_v1, v1, p1);
    int l2 = exp_mul(l_u1, u1, l_v0, v0, p2);
    exp_negate(l2, p2);
    int lr = exp_sum(l1, p1, l2, p2, r);
    return exp_sign(lr, r);
}

// ------------------------------------------------------------- FP64 stage
__device__ __noinline__ int orient3d_fp64_or_exact(float3 a, float3 b, float3 c, float3 d, PredCounters& pc) {
    // two coincident points make the determinant exactly zero
    if ((a.x == b.x && a.y == b.y && a.z == b.z) || (a.x == c.x && a.y == c.y && a.z == c.z) ||
        (a.x == d.x && a.y == d.y && a.z == d.z) || (b.x == c.x && b.y == c.y && b.z == c.z) ||
        (b.x == d.x && b.y == d.y && b.z == d.z) || (c.x == d.x && c.y == d.y && c.z == d.z))
        return 0;
    const double ux = (double)b.x - a.x, uy = (double)b.y - a.y, uz = (double)b.z - a.z;
    const double vx = (double)c.x - a.x, vy = (double)c.y - a.y, vz = (double)c.z - a.z;
    const double wx = (double)d.x - a.x, wy = (double)d.y - a.y, wz = (double)d.z - a.z;
    const double cx = vy * wz - vz * wy, cy = vz * wx - vx * wz, cz = vx * wy - vy * wx;
    const double det = ux * cx + uy * cy + uz * cz;
    const double perm = fabs(ux) * (fabs(vy * wz) + fabs(vz * wy)) + fabs(uy) * (fabs(vz * wx) + fabs(vx * wz)) +
                        fabs(uz) * (fabs(vx * wy) + fabs(vy * wx));
    const double bound = 12.0 * 1.1102230246251565e-16 * perm;
    if (det > bound) return 1;
    if (det < -bound) return -1;
    if (perm == 0.0) return 0;
    pc.fp64_ambiguous++;
    return orient3d_exact(a, b, c, d);
}

__device__ __noinline__ int orient2d_fp64_or_exact(float3 a, float3 b, float3 c, int i, int j, PredCounters& pc) {
    const double u0 = (double)fcomp(b, i) - fcomp(a, i), u1 = (double)fcomp(b, j) - fcomp(a, j);
    const double v0 = (double)fcomp(c, i) - fcomp(a, i), v1 = (double)fcomp(c, j) - fcomp(a, j);
    const double det = u0 * v1 - u1 * v0;
    const double perm = fabs(u0 * v1) + fabs(u1 * v0);
    const double bound = 8.0 * 1.1102230246251565e-16 * perm;
    if (det > bound) return 1;
    if (det < -bound) return -1;
    if (perm == 0.0) return 0;
    pc.fp64_ambiguous++;
    return orient2d_exact(a, b, c, i, j);
}

// ------------------------------------------------------------- FP32 stage
constexpr float kEps32 = 5.9604644775390625e-08f;  // 2^-24

__device__ __forceinline__ float3 f3sub(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 f3cross(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// |a| x |b| permanent vector: (|a_y b_z| + |a_z b_y|, ...)
__device__ __forceinline__ float3 f3cross_perm(float3 a, float3 b) {
    return make_float3(fabsf(a.y * b.z) + fabsf(a.z * b.y), fabsf(a.z * b.x) + fabsf(a.x * b.z),
                       fabsf(a.x * b.y) + fabsf(a.y * b.x));
}
__device__ __forceinline__ float f3dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float f3dot_abs(float3 a, float3 p) {
    return fabsf(a.x) * p.x + fabsf(a.y) * p.y + fabsf(a.z) * p.z;
}
// +1 / -1 when the float32 value's sign is certain, 0 when undecided.
// The bound is only valid without underflow or overflow, so tiny or huge
// permanents (and NaN) are always escalated to float64.
__device__ __forceinline__ int certain_sign(float v, float perm, float k) {
    if (!(perm >= 1e-30f && perm <= 1e36f)) return 0;
    const float bound = k * kEps32 * perm;
    return v > bound ? 1 : (v < -bound ? -1 : 0);
}

__device__ __forceinline__ bool same_point(float3 x, float3 y) { return x.x == y.x && x.y == y.y && x.z == y.z; }

// A segment endpoint that is a vertex of the triangle is a common point of
// the two closed sets (exact; covers shared vertices and shared edges).
__device__ __forceinline__ bool endpoint_is_vertex(float3 p, float3 q, float3 a, float3 b, float3 c) {
    return same_point(p, a) || same_point(p, b) || same_point(p, c) || same_point(q, a) || same_point(q, b) ||
           same_point(q, c);
}

__device__ __forceinline__ int orient3d_robust(float3 a, float3 b, float3 c, float3 d, PredCounters& pc) {
    const float3 u = f3sub(b, a), v = f3sub(c, a), w = f3sub(d, a);
    const float3 cr = f3cross(v, w), cp = f3cross_perm(v, w);
    int s = certain_sign(f3dot(u, cr), f3dot_abs(u, cp), 12.0f);
    if (s != 0) return s;
    pc.fp32_ambiguous++;
    return orient3d_fp64_or_exact(a, b, c, d, pc);
}

__device__ __forceinline__ int orient2d_robust(float3 a, float3 b, float3 c, int i, int j, PredCounters& pc) {
    const float u0 = fcomp(b, i) - fcomp(a, i), u1 = fcomp(b, j) - fcomp(a, j);
    const float v0 = fcomp(c, i) - fcomp(a, i), v1 = fcomp(c, j) - fcomp(a, j);
    const float t1 = u0 * v1, t2 = u1 * v0;
    int s = certain_sign(t1 - t2, fabsf(t1) + fabsf(t2), 8.0f);
    if (s != 0) return s;
    pc.fp32_ambiguous++;
    return orient2d_fp64_or_exact(a, b, c, i, j, pc);
}

// ------------------------------------------------------- coplanar fallback
__device__ __forceinline__ bool in_range(float v, float a, float b) { return fminf(a, b) <= v && v <= fmaxf(a, b); }
__device__ __forceinline__ bool on_seg_2d(float3 p, float3 q, float3 r, int i, int j) {
    return in_range(fcomp(r, i), fcomp(p, i), fcomp(q, i)) && in_range(fcomp(r, j), fcomp(p, j), fcomp(q, j));
}
__device__ __noinline__ bool segs_meet_2d(float3 p, float3 q, float3 u, float3 v, int i, int j, PredCounters& pc) {
    const int d1 = orient2d_robust(p, q, u, i, j, pc), d2 = orient2d_robust(p, q, v, i, j, pc);
    const int d3 = orient2d_robust(u, v, p, i, j, pc), d4 = orient2d_robust(u, v, q, i, j, pc);
    if (d1 * d2 < 0 && d3 * d4 < 0) return true;
    if (d1 == 0 && on_seg_2d(p, q, u, i, j)) return true;
    if (d2 == 0 && on_seg_2d(p, q, v, i, j)) return true;
    if (d3 == 0 && on_seg_2d(u, v, p, i, j)) return true;
    if (d4 == 0 && on_seg_2d(u, v, q, i, j)) return true;
    return false;
}
__device__ __noinline__ bool pt_in_tri_2d(float3 p, float3 a, float3 b, float3 c, int o, int i, int j,
                                          PredCounters& pc) {
    return orient2d_robust(a, b, p, i, j, pc) * o >= 0 && orient2d_robust(b, c, p, i, j, pc) * o >= 0 &&
           orient2d_robust(c, a, p, i, j, pc) * o >= 0;
}
__device__ __noinline__ bool seg_tri_coplanar(float3 p, float3 q, float3 a, float3 b, float3 c, PredCounters& pc) {
    const int nz = orient2d_robust(a, b, c, 0, 1, pc);
    const int nx = orient2d_robust(a, b, c, 1, 2, pc);
    const int ny = orient2d_robust(a, b, c, 2, 0, pc);
    int i, j, o;
    if (nz != 0) { i = 0; j = 1; o = nz; }
    else if (nx != 0) { i = 1; j = 2; o = nx; }
    else if (ny != 0) { i = 2; j = 0; o = ny; }
    else return false;  // zero-area triangle
    if (pt_in_tri_2d(p, a, b, c, o, i, j, pc) || pt_in_tri_2d(q, a, b, c, o, i, j, pc)) return true;
    return segs_meet_2d(p, q, a, b, i, j, pc) || segs_meet_2d(p, q, b, c, i, j, pc) ||
           segs_meet_2d(p, q, c, a, i, j, pc);
}

// ----------------------------------------------------------- the two tests

// Exact closed segment / closed triangle test with the FP32 filter.
__device__ __forceinline__ bool seg_tri_exact(float3 p, float3 q, float3 a, float3 b, float3 c, PredCounters& pc) {
    if (endpoint_is_vertex(p, q, a, b, c)) {
        // common point; only a zero-area triangle (empty by definition) is excluded
        if (orient2d_robust(a, b, c, 0, 1, pc) != 0 || orient2d_robust(a, b, c, 1, 2, pc) != 0 ||
            orient2d_robust(a, b, c, 2, 0, pc) != 0)
            return true;
        return false;
    }
    // Plane side of p and q: (p-a).n, (q-a).n with n = (b-a) x (c-a).
    const float3 u = f3sub(b, a), v = f3sub(c, a);
    const float3 n = f3cross(u, v), np = f3cross_perm(u, v);
    const float3 pa = f3sub(p, a), qa = f3sub(q, a);
    int sp = certain_sign(f3dot(pa, n), f3dot_abs(pa, np), 12.0f);
    int sq = certain_sign(f3dot(qa, n), f3dot_abs(qa, np), 12.0f);
    if (sp * sq > 0) return false;  // both certain, same side
    if (sp == 0) {
        pc.fp32_ambiguous++;
        sp = orient3d_fp64_or_exact(a, b, c, p, pc);
    }
    if (sq == 0) {
        pc.fp32_ambiguous++;
        sq = orient3d_fp64_or_exact(a, b, c, q, pc);
    }
    if (sp * sq > 0) return false;
    if (sp == 0 && sq == 0) return seg_tri_coplanar(p, q, a, b, c, pc);
    // The line pq meets the plane in one point; it is in the closed triangle
    // iff det[d, a-p, b-p], det[d, b-p, c-p], det[d, c-p, a-p] do not have
    // opposite strict signs (d = q - p).
    const float3 d = f3sub(q, p), A = f3sub(a, p), B = f3sub(b, p), C = f3sub(c, p);
    const float3 ma = f3cross(d, A), mpa = f3cross_perm(d, A);
    const float3 mb = f3cross(d, B), mpb = f3cross_perm(d, B);
    int s1 = certain_sign(f3dot(B, ma), f3dot_abs(B, mpa), 12.0f);   // det[d, A, B] = B.(d x A)
    int s2 = certain_sign(f3dot(C, mb), f3dot_abs(C, mpb), 12.0f);   // det[d, B, C] = C.(d x B)
    int s3 = certain_sign(-f3dot(C, ma), f3dot_abs(C, mpa), 12.0f);  // det[d, C, A] = -C.(d x A)
    if ((s1 > 0 || s2 > 0 || s3 > 0) && (s1 < 0 || s2 < 0 || s3 < 0)) return false;
    if (s1 == 0) {
        pc.fp32_ambiguous++;
        s1 = orient3d_fp64_or_exact(p, q, a, b, pc);
    }
    if (s2 == 0) {
        pc.fp32_ambiguous++;
        s2 = orient3d_fp64_or_exact(p, q, b, c, pc);
    }
    if (s3 == 0) {
        pc.fp32_ambiguous++;
        s3 = orient3d_fp64_or_exact(p, q, c, a, pc);
    }
    const bool pos = s1 > 0 || s2 > 0 || s3 > 0, neg = s1 < 0 || s2 < 0 || s3 < 0;
    if (pos && neg) return false;
    if (!pos && !neg) return false;  // only for a zero-area triangle
    return true;
}

// Float32-only classification of the closed segment / triangle test:
// SEG_MISS and SEG_HIT are certain (the same answer as seg_tri_exact);
// SEG_AMBIGUOUS means the float32 bound could not decide and the exact test
// must be run.
enum SegClass { SEG_MISS = 0, SEG_HIT = 1, SEG_AMBIGUOUS = 2 };

__device__ __forceinline__ int seg_tri_fp32_class(float3 p, float3 q, float3 a, float3 b, float3 c) {
    if (endpoint_is_vertex(p, q, a, b, c)) {
        // a common point, unless the triangle has zero area (then it is empty)
        const float3 u0 = f3sub(b, a), v0 = f3sub(c, a);
        const float3 n0 = f3cross(u0, v0), np0 = f3cross_perm(u0, v0);
        if (certain_sign(n0.x, np0.x, 8.0f) != 0 || certain_sign(n0.y, np0.y, 8.0f) != 0 ||
            certain_sign(n0.z, np0.z, 8.0f) != 0)
            return SEG_HIT;
        return SEG_AMBIGUOUS;
    }
    const float3 u = f3sub(b, a), v = f3sub(c, a);
    const float3 n = f3cross(u, v), np = f3cross_perm(u, v);
    const float3 pa = f3sub(p, a), qa = f3sub(q, a);
    const int sp = certain_sign(f3dot(pa, n), f3dot_abs(pa, np), 12.0f);
    const int sq = certain_sign(f3dot(qa, n), f3dot_abs(qa, np), 12.0f);
    if (sp * sq > 0) return SEG_MISS;
    if (sp == 0 || sq == 0) return SEG_AMBIGUOUS;
    const float3 d = f3sub(q, p), A = f3sub(a, p), B = f3sub(b, p), C = f3sub(c, p);
    const float3 ma = f3cross(d, A), mpa = f3cross_perm(d, A);
    const float3 mb = f3cross(d, B), mpb = f3cross_perm(d, B);
    const int s1 = certain_sign(f3dot(B, ma), f3dot_abs(B, mpa), 12.0f);
    const int s2 = certain_sign(f3dot(C, mb), f3dot_abs(C, mpb), 12.0f);
    const int s3 = certain_sign(-f3dot(C, ma), f3dot_abs(C, mpa), 12.0f);
    if ((s1 > 0 || s2 > 0 || s3 > 0) && (s1 < 0 || s2 < 0 || s3 < 0)) return SEG_MISS;
    if (s1 == 0 || s2 == 0 || s3 == 0) return SEG_AMBIGUOUS;
    return SEG_HIT;
}

// Plain float32 Moller-Trumbore on the segment p->q (no fallback).
__device__ __forceinline__ bool seg_tri_mt_fp32(float3 p, float3 q, float3 a, float3 b, float3 c) {
    const float e1x = __fsub_rn(b.x, a.x), e1y = __fsub_rn(b.y, a.y), e1z = __fsub_rn(b.z, a.z);
    const float e2x = __fsub_rn(c.x, a.x), e2y = __fsub_rn(c.y, a.y), e2z = __fsub_rn(c.z, a.z);
    const float dx = __fsub_rn(q.x, p.x), dy = __fsub_rn(q.y, p.y), dz = __fsub_rn(q.z, p.z);
    const float pvx = __fsub_rn(__fmul_rn(dy, e2z), __fmul_rn(dz, e2y));
    const float pvy = __fsub_rn(__fmul_rn(dz, e2x), __fmul_rn(dx, e2z));
    const float pvz = __fsub_rn(__fmul_rn(dx, e2y), __fmul_rn(dy, e2x));
    const float det = __fadd_rn(__fadd_rn(__fmul_rn(e1x, pvx), __fmul_rn(e1y, pvy)), __fmul_rn(e1z, pvz));
    if (det == 0.0f) return false;
    const float sx = __fsub_rn(p.x, a.x), sy = __fsub_rn(p.y, a.y), sz = __fsub_rn(p.z, a.z);
    const float u = __fadd_rn(__fadd_rn(__fmul_rn(sx, pvx), __fmul_rn(sy, pvy)), __fmul_rn(sz, pvz));
    const float qvx = __fsub_rn(__fmul_rn(sy, e1z), __fmul_rn(sz, e1y));
    const float qvy = __fsub_rn(__fmul_rn(sz, e1x), __fmul_rn(sx, e1z));
    const float qvz = __fsub_rn(__fmul_rn(sx, e1y), __fmul_rn(sy, e1x));
    const float v = __fadd_rn(__fadd_rn(__fmul_rn(dx, qvx), __fmul_rn(dy, qvy)), __fmul_rn(dz, qvz));
    const float t = __fadd_rn(__fadd_rn(__fmul_rn(e2x, qvx), __fmul_rn(e2y, qvy)), __fmul_rn(e2z, qvz));
    const float uv = __fadd_rn(u, v);
    if (det > 0.0f) return u >= 0.0f && v >= 0.0f && uv <= det && t >= 0.0f && t <= det;
    return u <= 0.0f && v <= 0.0f && uv >= det && t <= 0.0f && t >= det;
}

// Symbolic tie-break of orient2d(u, v, p) = 0 for p + (eps, eps^2).
__device__ __forceinline__ int sos_edge_sign(float3 u, float3 v) {
    if (u.y != v.y) return u.y > v.y ? 1 : -1;
    if (v.x != u.x) return v.x > u.x ? 1 : -1;
    return 0;
}

__device__ __forceinline__ bool zray_cross(float3 p, float3 a, float3 b, float3 c, PredCounters& pc) {
    const int o = orient2d_robust(a, b, c, 0, 1, pc);
    if (o == 0) return false;
    int s = orient2d_robust(a, b, p, 0, 1, pc);
    if (s == 0) s = sos_edge_sign(a, b);
    if (s != o) return false;
    s = orient2d_robust(b, c, p, 0, 1, pc);
    if (s == 0) s = sos_edge_sign(b, c);
    if (s != o) return false;
    s = orient2d_robust(c, a, p, 0, 1, pc);
    if (s == 0) s = sos_edge_sign(c, a);
    if (s != o) return false;
    return orient3d_robust(a, b, c, p, pc) == -o;
}

}  // namespace pgpu
