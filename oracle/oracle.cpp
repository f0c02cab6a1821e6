// CPU oracle for the Pierce mesh-join path — TEST INFRASTRUCTURE ONLY.
//
// This file restates, on the CPU and with exact arithmetic, the pair sets the
// reference's join executables define.  It is the checker for the CUDA path:
// only tests, the smoke check and the CPU-baseline leg of the benchmark load
// it, and no product code path may call it.
//
// Semantics (reference file:line in the Pierce project):
//  * overlap pair set S_surf: (a, b) such that a closed unique-edge segment of
//    object a meets a closed triangle of object b, or an edge of b meets a
//    triangle of a.  This is the edge-ray overlap of
//    pierce/query/src/cuda/mesh_overlap_edges.cu:105-208 (every unique edge,
//    both directions, pair order kept as (A-object, B-object) via
//    swap_pair_order) with its floating-point hit test replaced by exact
//    predicates; for closed triangles it equals the Face baseline's
//    "some triangle of a intersects some triangle of b"
//    (baselines/face/src/overlap_query.cpp:163-177), because two closed
//    triangles meet iff an edge of one meets the other.
//  * parity pairs: the first vertex of a source object (vertex x of its
//    lowest-index triangle, pierce/query/src/applications/
//    pierce_containment_main.cpp:336-347) casts a +Z ray; (src, tgt) is
//    emitted when the ray crosses tgt's triangles an odd number of times
//    (pierce/query/src/cuda/mesh_intersection_anyhit.cu:46-240,
//    mesh_containment.cu:179-293).  Crossings are decided exactly: the
//    query point is perturbed symbolically by (eps, eps^2) in x, y so that it
//    never lies on a projected edge or vertex, vertical triangles are never
//    crossed, and a triangle counts only if it lies strictly above the point.
//  * intersection = S_surf U parity(A in B) U parity(B in A)
//    (pierce_intersection_main.cpp:78-177); containment = parity(B in A)
//    minus S_surf (pierce_containment_main.cpp:385-550).
//  * FP32 plain form: the Moller-Trumbore segment test evaluated in float32
//    with a fixed operation order and no fused multiply-add, applied to every
//    triangle whose bounding box meets the segment's bounding box.  Used to
//    count the mismatches of an unguarded float32 filter.
//
// Exact arithmetic: every float32 is an integer multiple of 2^-173 below
// 2^301, so each predicate is the sign of a polynomial in exact integers.
// Evaluation first uses double precision with a generous forward error bound
// and falls back to a 1280-bit two's-complement integer evaluation when the
// double result is within the bound.  (The CUDA path uses a different exact
// method — floating-point expansions — so the two are independent.)
//
// Zero-area triangles (all three coordinate-plane projections collinear) are
// treated as empty by every test here, as by the CUDA path.
#include <algorithm>
#include <limits>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- bigint --
constexpr int kLimbs = 20;  // 1280 bits

struct Big {
    uint64_t w[kLimbs];
};

inline void big_zero(Big& r) { std::memset(r.w, 0, sizeof(r.w)); }
inline bool big_neg(const Big& a) { return (a.w[kLimbs - 1] >> 63) != 0; }
inline bool big_is_zero(const Big& a) {
    for (int i = 0; i < kLimbs; ++i)
        if (a.w[i]) return false;
    return true;
}
inline int big_sign(const Big& a) { return big_neg(a) ? -1 : (big_is_zero(a) ? 0 : 1); }

inline void big_add(const Big& a, const Big& b, Big& r) {
    unsigned __int128 carry = 0;
    for (int i = 0; i < kLimbs; ++i) {
        unsigned __int128 s = (unsigned __int128)a.w[i] + b.w[i] + carry;
        r.w[i] = (uint64_t)s;
        carry = s >> 64;
    }
}
inline void big_negate(const Big& a, Big& r) {
    unsigned __int128 carry = 1;
    for (int i = 0; i < kLimbs; ++i) {
        unsigned __int128 s = (unsigned __int128)(~a.w[i]) + carry;
        r.w[i] = (uint64_t)s;
        carry = s >> 64;
    }
}
inline void big_sub(const Big& a, const Big& b, Big& r) {
    Big nb;
    big_negate(b, nb);
    big_add(a, nb, r);
}
inline void big_mul(const Big& a, const Big& b, Big& r) {
    Big ma = a, mb = b;
    bool na = big_neg(a), nb = big_neg(b);
    if (na) big_negate(a, ma);
    if (nb) big_negate(b, mb);
    int la = kLimbs, lb = kLimbs;
    while (la > 0 && ma.w[la - 1] == 0) --la;
    while (lb > 0 && mb.w[lb - 1] == 0) --lb;
    Big p;
    big_zero(p);
    for (int i = 0; i < la; ++i) {
        unsigned __int128 carry = 0;
        for (int j = 0; j < lb && i + j < kLimbs; ++j) {
            unsigned __int128 t = (unsigned __int128)ma.w[i] * mb.w[j] + p.w[i + j] + carry;
            p.w[i + j] = (uint64_t)t;
            carry = t >> 64;
        }
        if (i + lb < kLimbs) p.w[i + lb] = (uint64_t)carry;
    }
    if (na != nb) big_negate(p, r);
    else r = p;
}
// Exact value of a float32 scaled by 2^173.
inline void big_from_float(float f, Big& r) {
    big_zero(r);
    if (f == 0.0f) return;
    int ex = 0;
    double fr = std::frexp((double)f, &ex);          // f = fr * 2^ex, |fr| in [0.5, 1)
    int64_t m = (int64_t)std::ldexp(fr, 24);          // exact 24-bit mantissa
    int shift = ex - 24 + 173;                        // >= 0 for every float32
    bool neg = m < 0;
    uint64_t mag = (uint64_t)(neg ? -m : m);
    int limb = shift / 64, bit = shift % 64;
    r.w[limb] = mag << bit;
    if (bit && limb + 1 < kLimbs) r.w[limb + 1] = mag >> (64 - bit);
    if (neg) big_negate(r, r);
}

// ------------------------------------------------------------- predicates --
struct P3 {
    float x, y, z;
};
inline float comp(const P3& p, int k) { return k == 0 ? p.x : (k == 1 ? p.y : p.z); }

std::atomic<uint64_t> g_exact_calls{0};

// det[b-a, c-a, d-a], exact, scaled by 2^(3 * 173)
void orient3d_value(const P3& a, const P3& b, const P3& c, const P3& d, Big& s) {
    Big A[3], B[3], C[3], D[3];
    for (int k = 0; k < 3; ++k) {
        big_from_float(comp(a, k), A[k]);
        big_from_float(comp(b, k), B[k]);
        big_from_float(comp(c, k), C[k]);
        big_from_float(comp(d, k), D[k]);
    }
    Big u[3], v[3], w[3];
    for (int k = 0; k < 3; ++k) {
        big_sub(B[k], A[k], u[k]);
        big_sub(C[k], A[k], v[k]);
        big_sub(D[k], A[k], w[k]);
    }
    // det = u . (v x w)
    Big t1, t2, cx, cy, cz, r;
    big_mul(v[1], w[2], t1); big_mul(v[2], w[1], t2); big_sub(t1, t2, cx);
    big_mul(v[2], w[0], t1); big_mul(v[0], w[2], t2); big_sub(t1, t2, cy);
    big_mul(v[0], w[1], t1); big_mul(v[1], w[0], t2); big_sub(t1, t2, cz);
    big_mul(u[0], cx, s);
    big_mul(u[1], cy, t1); big_add(s, t1, r);
    big_mul(u[2], cz, t1); big_add(r, t1, s);
}

// sign of det[b-a, c-a, d-a]
int orient3d_exact(const P3& a, const P3& b, const P3& c, const P3& d) {
    Big s;
    orient3d_value(a, b, c, d, s);
    return big_sign(s);
}

int orient3d(const P3& a, const P3& b, const P3& c, const P3& d) {
    const double ux = (double)b.x - a.x, uy = (double)b.y - a.y, uz = (double)b.z - a.z;
    const double vx = (double)c.x - a.x, vy = (double)c.y - a.y, vz = (double)c.z - a.z;
    const double wx = (double)d.x - a.x, wy = (double)d.y - a.y, wz = (double)d.z - a.z;
    const double cx = vy * wz - vz * wy, cy = vz * wx - vx * wz, cz = vx * wy - vy * wx;
    const double det = ux * cx + uy * cy + uz * cz;
    const double perm = std::fabs(ux) * (std::fabs(vy * wz) + std::fabs(vz * wy)) +
                        std::fabs(uy) * (std::fabs(vz * wx) + std::fabs(vx * wz)) +
                        std::fabs(uz) * (std::fabs(vx * wy) + std::fabs(vy * wx));
    const double bound = 1e-14 * perm;
    if (det > bound) return 1;
    if (det < -bound) return -1;
    if (perm == 0.0) return 0;
    g_exact_calls.fetch_add(1, std::memory_order_relaxed);
    return orient3d_exact(a, b, c, d);
}

// sign of (b_i - a_i)(c_j - a_j) - (b_j - a_j)(c_i - a_i) on coordinate axes (i, j)
int orient2d_exact(const P3& a, const P3& b, const P3& c, int i, int j) {
    Big ai, aj, bi, bj, ci, cj;
    big_from_float(comp(a, i), ai); big_from_float(comp(a, j), aj);
    big_from_float(comp(b, i), bi); big_from_float(comp(b, j), bj);
    big_from_float(comp(c, i), ci); big_from_float(comp(c, j), cj);
    Big u0, u1, v0, v1, t1, t2, r;
    big_sub(bi, ai, u0); big_sub(bj, aj, u1);
    big_sub(ci, ai, v0); big_sub(cj, aj, v1);
    big_mul(u0, v1, t1); big_mul(u1, v0, t2); big_sub(t1, t2, r);
    return big_sign(r);
}

int orient2d(const P3& a, const P3& b, const P3& c, int i, int j) {
    const double u0 = (double)comp(b, i) - comp(a, i), u1 = (double)comp(b, j) - comp(a, j);
    const double v0 = (double)comp(c, i) - comp(a, i), v1 = (double)comp(c, j) - comp(a, j);
    const double det = u0 * v1 - u1 * v0;
    const double perm = std::fabs(u0 * v1) + std::fabs(u1 * v0);
    const double bound = 1e-14 * perm;
    if (det > bound) return 1;
    if (det < -bound) return -1;
    if (perm == 0.0) return 0;
    g_exact_calls.fetch_add(1, std::memory_order_relaxed);
    return orient2d_exact(a, b, c, i, j);
}

// Normal-vector signs of triangle abc: (n_x, n_y, n_z) = orient2d on (y,z), (z,x), (x,y).
inline void normal_signs(const P3& a, const P3& b, const P3& c, int s[3]) {
    s[0] = orient2d(a, b, c, 1, 2);
    s[1] = orient2d(a, b, c, 2, 0);
    s[2] = orient2d(a, b, c, 0, 1);
}

inline bool between(float v, float lo, float hi) { return lo <= v && v <= hi; }

// Closed collinear point-on-segment check in the (i, j) plane.
inline bool on_segment_2d(const P3& p, const P3& q, const P3& r, int i, int j) {
    return between(comp(r, i), std::min(comp(p, i), comp(q, i)), std::max(comp(p, i), comp(q, i))) &&
           between(comp(r, j), std::min(comp(p, j), comp(q, j)), std::max(comp(p, j), comp(q, j)));
}

bool segments_meet_2d(const P3& p, const P3& q, const P3& u, const P3& v, int i, int j) {
    const int d1 = orient2d(p, q, u, i, j), d2 = orient2d(p, q, v, i, j);
    const int d3 = orient2d(u, v, p, i, j), d4 = orient2d(u, v, q, i, j);
    if (d1 * d2 < 0 && d3 * d4 < 0) return true;
    if (d1 == 0 && on_segment_2d(p, q, u, i, j)) return true;
    if (d2 == 0 && on_segment_2d(p, q, v, i, j)) return true;
    if (d3 == 0 && on_segment_2d(u, v, p, i, j)) return true;
    if (d4 == 0 && on_segment_2d(u, v, q, i, j)) return true;
    return false;
}

bool point_in_triangle_2d(const P3& p, const P3& a, const P3& b, const P3& c, int o, int i, int j) {
    const int s1 = orient2d(a, b, p, i, j), s2 = orient2d(b, c, p, i, j), s3 = orient2d(c, a, p, i, j);
    return s1 * o >= 0 && s2 * o >= 0 && s3 * o >= 0;
}

struct Box {
    float lo[3], hi[3];
};
inline Box seg_box(const P3& p, const P3& q) {
    Box b;
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = std::min(comp(p, k), comp(q, k));
        b.hi[k] = std::max(comp(p, k), comp(q, k));
    }
    return b;
}
inline Box tri_box(const P3& a, const P3& b, const P3& c) {
    Box r;
    for (int k = 0; k < 3; ++k) {
        r.lo[k] = std::min(comp(a, k), std::min(comp(b, k), comp(c, k)));
        r.hi[k] = std::max(comp(a, k), std::max(comp(b, k), comp(c, k)));
    }
    return r;
}
inline bool boxes_overlap(const Box& a, const Box& b) {
    for (int k = 0; k < 3; ++k)
        if (a.hi[k] < b.lo[k] || b.hi[k] < a.lo[k]) return false;
    return true;
}

// Exact: does the closed segment pq meet the closed triangle abc?
bool seg_tri_exact(const P3& p, const P3& q, const P3& a, const P3& b, const P3& c) {
    const int sp = orient3d(a, b, c, p), sq = orient3d(a, b, c, q);
    if (sp * sq > 0) return false;
    if (sp == 0 && sq == 0) {
        int n[3];
        normal_signs(a, b, c, n);
        int i, j, o;
        if (n[2] != 0) { i = 0; j = 1; o = n[2]; }
        else if (n[0] != 0) { i = 1; j = 2; o = n[0]; }
        else if (n[1] != 0) { i = 2; j = 0; o = n[1]; }
        else return false;  // zero-area triangle
        if (point_in_triangle_2d(p, a, b, c, o, i, j) || point_in_triangle_2d(q, a, b, c, o, i, j)) return true;
        return segments_meet_2d(p, q, a, b, i, j) || segments_meet_2d(p, q, b, c, i, j) ||
               segments_meet_2d(p, q, c, a, i, j);
    }
    // Line pq crosses (or touches) the plane at a single point; it lies in
    // the closed triangle iff the three edge orientations do not disagree.
    const int s1 = orient3d(p, q, a, b), s2 = orient3d(p, q, b, c), s3 = orient3d(p, q, c, a);
    // orient3d(p,q,u,v) = sign det[q-p, u-p, v-p]; a common sign factor
    // does not matter.
    const bool has_pos = s1 > 0 || s2 > 0 || s3 > 0;
    const bool has_neg = s1 < 0 || s2 < 0 || s3 < 0;
    if (has_pos && has_neg) return false;
    if (!has_pos && !has_neg) {
        // All zero: only possible for a zero-area triangle.
        int n[3];
        normal_signs(a, b, c, n);
        if (n[0] == 0 && n[1] == 0 && n[2] == 0) return false;
        return true;
    }
    return true;
}

// Exact +Z ray crossing with the symbolic (eps, eps^2) perturbation of p.
inline int sos_edge_sign(const P3& u, const P3& v) {
    if (u.y != v.y) return u.y > v.y ? 1 : -1;
    if (v.x != u.x) return v.x > u.x ? 1 : -1;
    return 0;
}
bool zray_crosses(const P3& p, const P3& a, const P3& b, const P3& c) {
    const int o = orient2d(a, b, c, 0, 1);
    if (o == 0) return false;
    const P3* e[3][2] = {{&a, &b}, {&b, &c}, {&c, &a}};
    for (auto& ed : e) {
        int s = orient2d(*ed[0], *ed[1], p, 0, 1);
        if (s == 0) s = sos_edge_sign(*ed[0], *ed[1]);
        if (s != o) return false;
    }
    const int d = orient3d(a, b, c, p);
    return d == -o;
}

// Float32 Moller-Trumbore on segment p->q, fixed operation order, no FMA
// (this file is compiled with -ffp-contract=off).
bool seg_tri_mt_fp32(const P3& p, const P3& q, const P3& a, const P3& b, const P3& c) {
    const float e1x = b.x - a.x, e1y = b.y - a.y, e1z = b.z - a.z;
    const float e2x = c.x - a.x, e2y = c.y - a.y, e2z = c.z - a.z;
    const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
    const float pvx = dy * e2z - dz * e2y, pvy = dz * e2x - dx * e2z, pvz = dx * e2y - dy * e2x;
    const float det = (e1x * pvx + e1y * pvy) + e1z * pvz;
    if (det == 0.0f) return false;
    const float sx = p.x - a.x, sy = p.y - a.y, sz = p.z - a.z;
    const float u = (sx * pvx + sy * pvy) + sz * pvz;
    const float qvx = sy * e1z - sz * e1y, qvy = sz * e1x - sx * e1z, qvz = sx * e1y - sy * e1x;
    const float v = (dx * qvx + dy * qvy) + dz * qvz;
    const float t = (e2x * qvx + e2y * qvy) + e2z * qvz;
    const float uv = u + v;
    if (det > 0.0f) return u >= 0.0f && v >= 0.0f && uv <= det && t >= 0.0f && t <= det;
    return u <= 0.0f && v <= 0.0f && uv >= det && t <= 0.0f && t >= det;
}

// --------------------------------------------------------------- CPU BVH --
struct Mesh {
    const float* v;
    const uint32_t* idx;
    const int32_t* obj;
    uint64_t nt;
    P3 vert(uint32_t i) const { return P3{v[3 * (size_t)i], v[3 * (size_t)i + 1], v[3 * (size_t)i + 2]}; }
    void tri(uint64_t t, P3& a, P3& b, P3& c) const {
        a = vert(idx[3 * t]);
        b = vert(idx[3 * t + 1]);
        c = vert(idx[3 * t + 2]);
    }
};

struct BvhNode {
    Box box;
    int64_t left;   // >= 0: child node index; < 0: leaf
    uint64_t first, count;
};

struct Bvh {
    std::vector<BvhNode> nodes;
    std::vector<uint64_t> order;
    std::vector<Box> boxes;

    void build(const Mesh& m) {
        boxes.resize(m.nt);
        order.resize(m.nt);
        std::vector<float> cen(3 * m.nt);
        for (uint64_t t = 0; t < m.nt; ++t) {
            P3 a, b, c;
            m.tri(t, a, b, c);
            boxes[t] = tri_box(a, b, c);
            for (int k = 0; k < 3; ++k) cen[3 * t + k] = 0.5f * (boxes[t].lo[k] + boxes[t].hi[k]);
            order[t] = t;
        }
        nodes.clear();
        if (m.nt == 0) return;
        nodes.reserve(2 * m.nt / 4 + 2);
        struct Task {
            uint64_t node, first, count;
        };
        nodes.push_back(BvhNode{});
        std::vector<Task> stack{{0, 0, m.nt}};
        while (!stack.empty()) {
            Task tk = stack.back();
            stack.pop_back();
            Box bb{{1e38f, 1e38f, 1e38f}, {-1e38f, -1e38f, -1e38f}};
            float clo[3] = {1e38f, 1e38f, 1e38f}, chi[3] = {-1e38f, -1e38f, -1e38f};
            for (uint64_t i = tk.first; i < tk.first + tk.count; ++i) {
                const Box& b = boxes[order[i]];
                for (int k = 0; k < 3; ++k) {
                    bb.lo[k] = std::min(bb.lo[k], b.lo[k]);
                    bb.hi[k] = std::max(bb.hi[k], b.hi[k]);
                    clo[k] = std::min(clo[k], cen[3 * order[i] + k]);
                    chi[k] = std::max(chi[k], cen[3 * order[i] + k]);
                }
            }
            BvhNode& n = nodes[tk.node];
            n.box = bb;
            if (tk.count <= 4) {
                n.left = -1;
                n.first = tk.first;
                n.count = tk.count;
                continue;
            }
            int axis = 0;
            for (int k = 1; k < 3; ++k)
                if (chi[k] - clo[k] > chi[axis] - clo[axis]) axis = k;
            uint64_t mid = tk.first + tk.count / 2;
            std::nth_element(order.begin() + tk.first, order.begin() + mid, order.begin() + tk.first + tk.count,
                             [&](uint64_t x, uint64_t y) { return cen[3 * x + axis] < cen[3 * y + axis]; });
            uint64_t l = nodes.size();
            nodes.push_back(BvhNode{});
            nodes.push_back(BvhNode{});
            nodes[tk.node].left = (int64_t)l;
            stack.push_back({l, tk.first, mid - tk.first});
            stack.push_back({l + 1, mid, tk.first + tk.count - mid});
        }
    }

    template <class Overlap, class Visit>
    void query(Overlap overlap, Visit visit) const {
        if (nodes.empty()) return;
        uint64_t stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp) {
            const BvhNode& n = nodes[stack[--sp]];
            if (!overlap(n.box)) continue;
            if (n.left < 0) {
                for (uint64_t i = n.first; i < n.first + n.count; ++i)
                    if (overlap(boxes[order[i]])) visit(order[i]);
            } else {
                stack[sp++] = (uint64_t)n.left;
                stack[sp++] = (uint64_t)n.left + 1;
            }
        }
    }
};

inline uint64_t pack(int32_t a, int32_t b) { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; }

void sort_unique(std::vector<uint64_t>& k) {
    std::sort(k.begin(), k.end());
    k.erase(std::unique(k.begin(), k.end()), k.end());
}

uint64_t* to_malloc(const std::vector<uint64_t>& v, uint64_t* n) {
    *n = v.size();
    uint64_t* out = (uint64_t*)std::malloc(std::max<size_t>(1, v.size()) * sizeof(uint64_t));
    if (out && !v.empty()) std::memcpy(out, v.data(), v.size() * sizeof(uint64_t));
    return out;
}

// Edge rays of `src` against triangles of `tgt`; pairs (srcObj, tgtObj),
// swapped when swap != 0.  mode 0: exact, 1: float32 Moller-Trumbore.
void edge_join(const float* es, const float* ee, const int32_t* esrc, uint64_t ne, const Mesh& tgt,
               const Bvh& bvh, int swap, int mode, std::vector<uint64_t>& out, uint64_t* tests) {
    int nth = 1;
#ifdef _OPENMP
    nth = omp_get_max_threads();
#endif
    std::vector<std::vector<uint64_t>> per(nth);
    std::vector<uint64_t> cnt(nth, 0);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t e = 0; e < (int64_t)ne; ++e) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        const P3 p{es[3 * e], es[3 * e + 1], es[3 * e + 2]};
        const P3 q{ee[3 * e], ee[3 * e + 1], ee[3 * e + 2]};
        const Box sb = seg_box(p, q);
        const int32_t so = esrc[e];
        int32_t last = -1;
        bvh.query([&](const Box& b) { return boxes_overlap(sb, b); },
                  [&](uint64_t t) {
                      const int32_t to = tgt.obj[t];
                      if (to == last) return;
                      P3 a, b, c;
                      tgt.tri(t, a, b, c);
                      cnt[tid]++;
                      const bool hit = mode == 0 ? seg_tri_exact(p, q, a, b, c) : seg_tri_mt_fp32(p, q, a, b, c);
                      if (hit) {
                          last = to;
                          per[tid].push_back(swap ? pack(to, so) : pack(so, to));
                      }
                  });
    }
    for (auto& v : per) out.insert(out.end(), v.begin(), v.end());
    if (tests)
        for (uint64_t c : cnt) *tests += c;
}

// The reference's edge-ray semantics (pierce/query/src/cuda/
// mesh_overlap_edges.cu:105-176) on exact hits: the ray starts at the edge's
// start point with tmin = nextafterf(0), so a hit there is not seen; a ray in
// a triangle's plane is parallel to it and misses; each closest-hit
// iteration reports one hit and moves tmin past its t, so hits at one t
// count once (here the lowest target object wins the tie; the reference's
// winner depends on its traversal order); at most max_iter iterations
// report.  Hit parameters t = D(p) / (D(p) - D(q)), D(x) = det[b-a, c-a,
// x-a], are exact rationals compared by cross-multiplication (exact for
// coordinates below 2^20 in magnitude).  A zero-length edge reports nothing.
struct RefHit {
    Big num, den;  // t = num / den, den > 0
    int32_t obj;
};

bool ref_t_less(const RefHit& x, const RefHit& y) {
    Big l, r, d;
    big_mul(x.num, y.den, l);
    big_mul(y.num, x.den, r);
    big_sub(l, r, d);
    return big_neg(d);
}

bool ref_t_equal(const RefHit& x, const RefHit& y) {
    Big l, r, d;
    big_mul(x.num, y.den, l);
    big_mul(y.num, x.den, r);
    big_sub(l, r, d);
    return big_is_zero(d);
}

void edge_join_reference(const float* es, const float* ee, const int32_t* esrc, uint64_t ne, const Mesh& tgt,
                         const Bvh& bvh, int swap, int max_iter, std::vector<uint64_t>& out) {
    int nth = 1;
#ifdef _OPENMP
    nth = omp_get_max_threads();
#endif
    std::vector<std::vector<uint64_t>> per(nth);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t e = 0; e < (int64_t)ne; ++e) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        const P3 p{es[3 * e], es[3 * e + 1], es[3 * e + 2]};
        const P3 q{ee[3 * e], ee[3 * e + 1], ee[3 * e + 2]};
        if (p.x == q.x && p.y == q.y && p.z == q.z) continue;
        const Box sb = seg_box(p, q);
        const int32_t so = esrc[e];
        std::vector<RefHit> hits;
        bvh.query([&](const Box& b) { return boxes_overlap(sb, b); },
                  [&](uint64_t t) {
                      P3 a, b, c;
                      tgt.tri(t, a, b, c);
                      if (!seg_tri_exact(p, q, a, b, c)) return;
                      RefHit h;
                      Big dq;
                      orient3d_value(a, b, c, p, h.num);
                      orient3d_value(a, b, c, q, dq);
                      if (big_is_zero(h.num)) return;  // in the plane (parallel ray) or at the start point
                      big_sub(h.num, dq, h.den);
                      if (big_neg(h.den)) {
                          big_negate(h.num, h.num);
                          big_negate(h.den, h.den);
                      }
                      h.obj = tgt.obj[t];
                      hits.push_back(h);
                  });
        std::sort(hits.begin(), hits.end(), [](const RefHit& x, const RefHit& y) {
            if (ref_t_less(x, y)) return true;
            if (ref_t_less(y, x)) return false;
            return x.obj < y.obj;
        });
        int iters = 0;
        for (size_t i = 0; i < hits.size(); ++i) {
            if (i > 0 && ref_t_equal(hits[i], hits[i - 1])) continue;
            if (++iters > max_iter) break;
            per[tid].push_back(swap ? pack(hits[i].obj, so) : pack(so, hits[i].obj));
        }
    }
    for (auto& v : per) out.insert(out.end(), v.begin(), v.end());
}

// Parity pairs: first vertex of each source object against target triangles.
void parity_join(const float* first_vertices, int32_t nsrc, const Mesh& tgt, const Bvh& bvh, int swap,
                 std::vector<uint64_t>& out) {
    int nth = 1;
#ifdef _OPENMP
    nth = omp_get_max_threads();
#endif
    std::vector<std::vector<uint64_t>> per(nth);
#pragma omp parallel for schedule(dynamic, 64)
    for (int32_t s = 0; s < nsrc; ++s) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        const P3 p{first_vertices[3 * s], first_vertices[3 * s + 1], first_vertices[3 * s + 2]};
        std::vector<int32_t> hits;
        bvh.query(
            [&](const Box& b) {
                return b.lo[0] <= p.x && p.x <= b.hi[0] && b.lo[1] <= p.y && p.y <= b.hi[1] && b.hi[2] >= p.z;
            },
            [&](uint64_t t) {
                P3 a, b, c;
                tgt.tri(t, a, b, c);
                if (zray_crosses(p, a, b, c)) hits.push_back(tgt.obj[t]);
            });
        std::sort(hits.begin(), hits.end());
        for (size_t i = 0; i < hits.size();) {
            size_t j = i;
            while (j < hits.size() && hits[j] == hits[i]) ++j;
            if ((j - i) & 1) per[tid].push_back(swap ? pack(hits[i], s) : pack(s, hits[i]));
            i = j;
        }
    }
    for (auto& v : per) out.insert(out.end(), v.begin(), v.end());
}

// Crossing counts of the parity rays: for every source object s and target
// object t that s's +Z ray crosses, the entry (s << 32 | t, crossings), in
// key order.  The diagnostics of --enable-tracking list, per source, the
// targets of odd count with their counts (mesh_intersection_anyhit.cu:108-146,
// hit counts gathered by __anyhit__ah_containment :194-240).
void parity_crossings(const float* first_vertices, int32_t nsrc, const Mesh& tgt, const Bvh& bvh,
                      std::vector<uint64_t>& out) {
    int nth = 1;
#ifdef _OPENMP
    nth = omp_get_max_threads();
#endif
    std::vector<std::vector<uint64_t>> per(nth);
#pragma omp parallel for schedule(dynamic, 64)
    for (int32_t s = 0; s < nsrc; ++s) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        const P3 p{first_vertices[3 * s], first_vertices[3 * s + 1], first_vertices[3 * s + 2]};
        std::vector<int32_t> hits;
        bvh.query(
            [&](const Box& b) {
                return b.lo[0] <= p.x && p.x <= b.hi[0] && b.lo[1] <= p.y && p.y <= b.hi[1] && b.hi[2] >= p.z;
            },
            [&](uint64_t t) {
                P3 a, b, c;
                tgt.tri(t, a, b, c);
                if (zray_crosses(p, a, b, c)) hits.push_back(tgt.obj[t]);
            });
        std::sort(hits.begin(), hits.end());
        for (size_t i = 0; i < hits.size();) {
            size_t j = i;
            while (j < hits.size() && hits[j] == hits[i]) ++j;
            per[tid].push_back(pack(s, hits[i]));
            per[tid].push_back((uint64_t)(j - i));
            i = j;
        }
    }
    std::vector<std::pair<uint64_t, uint64_t>> all;
    for (auto& v : per)
        for (size_t i = 0; i < v.size(); i += 2) all.emplace_back(v[i], v[i + 1]);
    std::sort(all.begin(), all.end());
    for (auto& e : all) {
        out.push_back(e.first);
        out.push_back(e.second);
    }
}

// ------------------------------------------------------------------ TOUCH --
// Node of the STR tree over A's objects: its box, its children (internal)
// or A objects (leaf), and the B objects assigned to it.
struct TouchNode {
    Box box;
    bool leaf = false;
    std::vector<int> kids;
    std::vector<int32_t> objs;
    std::vector<int32_t> assigned;
};

Box touch_empty_box() {
    Box b;
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = std::numeric_limits<float>::max();
        b.hi[k] = -std::numeric_limits<float>::max();
    }
    return b;
}

void touch_extend(Box& b, const Box& o) {
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = std::min(b.lo[k], o.lo[k]);
        b.hi[k] = std::max(b.hi[k], o.hi[k]);
    }
}

bool touch_overlaps(const Box& a, const Box& b) {
    for (int k = 0; k < 3; ++k)
        if (a.hi[k] < b.lo[k] || a.lo[k] > b.hi[k]) return false;
    return true;
}

// One STR level: items sorted by box centre along x, cut into Sx slabs,
// each slab sorted along y and cut into Sy runs, each run sorted along z
// and cut into groups of `fanout` consecutive items; P = ceil(n / fanout),
// Sx = ceil(P^(1/3)), Sy = ceil(sqrt(P / Sx)) (touch_query.cpp:125-163).
std::vector<std::vector<int>> str_groups(std::vector<int> items, const std::vector<Box>& box, int fanout) {
    const size_t n = items.size();
    const double P = (double)((n + fanout - 1) / fanout);
    const int Sx = (int)std::ceil(std::pow(P, 1.0 / 3.0));
    const int Sy = (int)std::ceil(std::sqrt(P / Sx));
    auto by = [&](int d) {
        return [&box, d](int x, int y) { return box[x].lo[d] + box[x].hi[d] < box[y].lo[d] + box[y].hi[d]; };
    };
    std::sort(items.begin(), items.end(), by(0));
    std::vector<std::vector<int>> groups;
    size_t ix = 0;
    int sx = Sx;
    while (ix < n) {
        const size_t end_x = std::min(n, ix + (n - ix + sx - 1) / sx);
        std::sort(items.begin() + ix, items.begin() + end_x, by(1));
        size_t iy = ix;
        int sy = Sy;
        while (iy < end_x) {
            const size_t end_y = std::min(end_x, iy + (end_x - iy + sy - 1) / sy);
            std::sort(items.begin() + iy, items.begin() + end_y, by(2));
            for (size_t iz = iy; iz < end_y;) {
                std::vector<int> g;
                for (int i = 0; i < fanout && iz < end_y; ++i, ++iz) g.push_back(items[iz]);
                groups.push_back(std::move(g));
            }
            --sy;
            iy = end_y;
        }
        --sx;
        ix = end_x;
    }
    return groups;
}

void touch_join(const Mesh& A, const Mesh& B, std::vector<uint64_t>& keys, uint64_t* candidates_out) {
    // object boxes and per-object triangle lists
    auto objects = [](const Mesh& m, std::vector<Box>& box, std::vector<std::vector<uint32_t>>& tris) {
        int32_t n = 0;
        for (uint64_t t = 0; t < m.nt; ++t) n = std::max(n, m.obj[t] + 1);
        box.assign((size_t)n, touch_empty_box());
        tris.assign((size_t)n, {});
        for (uint64_t t = 0; t < m.nt; ++t) {
            const int32_t o = m.obj[t];
            if (o < 0) continue;
            P3 a, b, c;
            m.tri(t, a, b, c);
            touch_extend(box[o], tri_box(a, b, c));
            tris[o].push_back((uint32_t)t);
        }
    };
    std::vector<Box> boxA, boxB;
    std::vector<std::vector<uint32_t>> trisA, trisB;
    objects(A, boxA, trisA);
    objects(B, boxB, trisB);
    // STR tree over A's objects with triangles, fanout 2
    std::vector<TouchNode> nodes;
    std::vector<Box> level_box;
    std::vector<int> level;
    {
        std::vector<int> items;
        for (size_t o = 0; o < boxA.size(); ++o)
            if (!trisA[o].empty()) items.push_back((int)o);
        if (items.empty()) {
            if (candidates_out) *candidates_out = 0;
            return;
        }
        for (auto& g : str_groups(items, boxA, 2)) {
            TouchNode leaf;
            leaf.leaf = true;
            leaf.box = touch_empty_box();
            for (int o : g) {
                leaf.objs.push_back(o);
                touch_extend(leaf.box, boxA[o]);
            }
            level.push_back((int)nodes.size());
            nodes.push_back(std::move(leaf));
        }
    }
    while (level.size() > 1) {
        level_box.resize(nodes.size());
        for (size_t i = 0; i < nodes.size(); ++i) level_box[i] = nodes[i].box;
        std::vector<int> next;
        for (auto& g : str_groups(level, level_box, 2)) {
            TouchNode parent;
            parent.box = touch_empty_box();
            for (int c : g) {
                parent.kids.push_back(c);
                touch_extend(parent.box, nodes[c].box);
            }
            next.push_back((int)nodes.size());
            nodes.push_back(std::move(parent));
        }
        level = std::move(next);
    }
    const int root = level.front();
    // B objects: down the tree while exactly one child's box meets theirs;
    // assigned where several do, or to the leaf reached (touch_query.cpp:221-253)
    for (size_t o = 0; o < boxB.size(); ++o) {
        if (trisB[o].empty() || !touch_overlaps(boxB[o], nodes[root].box)) continue;
        int p = root;
        bool assigned = false;
        while (!nodes[p].leaf) {
            int count = 0, only = -1;
            for (int c : nodes[p].kids)
                if (touch_overlaps(boxB[o], nodes[c].box)) {
                    ++count;
                    only = c;
                }
            if (count == 0) break;
            if (count > 1) {
                nodes[p].assigned.push_back((int32_t)o);
                assigned = true;
                break;
            }
            p = only;
        }
        if (!assigned && nodes[p].leaf) nodes[p].assigned.push_back((int32_t)o);
    }
    // candidates: per work node, its descendant leaves' A objects whose box
    // meets an assigned B object's box (touch_query.cpp:268-302)
    std::vector<std::pair<int32_t, int32_t>> cand;
    std::vector<int> stack;
    for (size_t w = 0; w < nodes.size(); ++w) {
        if (nodes[w].assigned.empty()) continue;
        stack.assign(1, (int)w);
        while (!stack.empty()) {
            const int n = stack.back();
            stack.pop_back();
            if (!nodes[n].leaf) {
                for (int c : nodes[n].kids) stack.push_back(c);
                continue;
            }
            for (int32_t b : nodes[w].assigned) {
                if (!touch_overlaps(boxB[b], nodes[n].box)) continue;
                for (int32_t a : nodes[n].objs)
                    if (touch_overlaps(boxB[b], boxA[a])) cand.emplace_back(a, b);
            }
        }
    }
    if (candidates_out) *candidates_out = cand.size();
    // per B object with candidates: a hierarchy over its triangles
    std::vector<int> need(boxB.size(), 0);
    for (auto& c : cand) need[c.second] = 1;
    std::vector<std::vector<uint32_t>> idxB(boxB.size());
    std::vector<std::vector<int32_t>> objB(boxB.size());
    std::vector<Bvh> bvhB(boxB.size());
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t o = 0; o < (int64_t)boxB.size(); ++o) {
        if (!need[o]) continue;
        for (uint32_t t : trisB[o])
            for (int k = 0; k < 3; ++k) idxB[o].push_back(B.idx[3 * (size_t)t + k]);
        objB[o].assign(trisB[o].size(), (int32_t)o);
        bvhB[o].build(Mesh{B.v, idxB[o].data(), objB[o].data(), trisB[o].size()});
    }
    // refinement: a candidate is a pair when a triangle of a meets b
    std::vector<uint8_t> hit(cand.size(), 0);
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t i = 0; i < (int64_t)cand.size(); ++i) {
        const int32_t a = cand[i].first, b = cand[i].second;
        const Mesh Bo{B.v, idxB[b].data(), objB[b].data(), trisB[b].size()};
        bool found = false;
        for (uint32_t t : trisA[a]) {
            P3 p, q, r;
            A.tri(t, p, q, r);
            const Box tb = tri_box(p, q, r);
            bvhB[b].query([&](const Box& bx) { return !found && boxes_overlap(tb, bx); },
                          [&](uint64_t u) {
                              if (found) return;
                              P3 d, e, f;
                              Bo.tri(u, d, e, f);
                              found = seg_tri_exact(p, q, d, e, f) || seg_tri_exact(q, r, d, e, f) ||
                                      seg_tri_exact(r, p, d, e, f) || seg_tri_exact(d, e, p, q, r) ||
                                      seg_tri_exact(e, f, p, q, r) || seg_tri_exact(f, d, p, q, r);
                          });
            if (found) break;
        }
        hit[i] = found ? 1 : 0;
    }
    for (size_t i = 0; i < cand.size(); ++i)
        if (hit[i]) keys.push_back(pack(cand[i].first, cand[i].second));
}

}  // namespace

// ------------------------------------------------------------ C interface --
extern "C" {

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

uint64_t oracle_exact_calls(void) { return g_exact_calls.load(); }

int oracle_orient3d(const float* a, const float* b, const float* c, const float* d) {
    return orient3d(P3{a[0], a[1], a[2]}, P3{b[0], b[1], b[2]}, P3{c[0], c[1], c[2]}, P3{d[0], d[1], d[2]});
}
int oracle_orient3d_exact(const float* a, const float* b, const float* c, const float* d) {
    return orient3d_exact(P3{a[0], a[1], a[2]}, P3{b[0], b[1], b[2]}, P3{c[0], c[1], c[2]},
                          P3{d[0], d[1], d[2]});
}
int oracle_orient2d_xy(const float* a, const float* b, const float* c) {
    return orient2d(P3{a[0], a[1], a[2]}, P3{b[0], b[1], b[2]}, P3{c[0], c[1], c[2]}, 0, 1);
}
int oracle_seg_tri(const float* p, const float* q, const float* a, const float* b, const float* c, int mode) {
    P3 P{p[0], p[1], p[2]}, Q{q[0], q[1], q[2]}, A{a[0], a[1], a[2]}, B{b[0], b[1], b[2]}, Cc{c[0], c[1], c[2]};
    if (mode == 1) return boxes_overlap(seg_box(P, Q), tri_box(A, B, Cc)) && seg_tri_mt_fp32(P, Q, A, B, Cc);
    return seg_tri_exact(P, Q, A, B, Cc);
}
int oracle_zray_crosses(const float* p, const float* a, const float* b, const float* c) {
    return zray_crosses(P3{p[0], p[1], p[2]}, P3{a[0], a[1], a[2]}, P3{b[0], b[1], b[2]}, P3{c[0], c[1], c[2]});
}

// Overlap pairs (A-object, B-object), sorted ascending by (a << 32 | b).
// direction: 0 both, 1 A-edges vs B only, 2 B-edges vs A only.
// mode: 0 exact, 1 float32 Moller-Trumbore plain form.
uint64_t* oracle_overlap_pairs(const float* av, const uint32_t* ai, const int32_t* ao, uint64_t ant,
                               const float* aes, const float* aee, const int32_t* aesrc, uint64_t ane,
                               const float* bv, const uint32_t* bi, const int32_t* bo, uint64_t bnt,
                               const float* bes, const float* bee, const int32_t* besrc, uint64_t bne,
                               int direction, int mode, uint64_t* n_out, uint64_t* tests_out) {
    Mesh A{av, ai, ao, ant}, B{bv, bi, bo, bnt};
    std::vector<uint64_t> keys;
    uint64_t tests = 0;
    if (direction == 0 || direction == 1) {
        Bvh bb;
        bb.build(B);
        edge_join(aes, aee, aesrc, ane, B, bb, 0, mode, keys, &tests);
    }
    if (direction == 0 || direction == 2) {
        Bvh ab;
        ab.build(A);
        edge_join(bes, bee, besrc, bne, A, ab, 1, mode, keys, &tests);
    }
    sort_unique(keys);
    if (tests_out) *tests_out = tests;
    return to_malloc(keys, n_out);
}

// Overlap pairs under the reference's edge-ray semantics (see
// edge_join_reference), sorted like oracle_overlap_pairs.
uint64_t* oracle_overlap_pairs_reference(const float* av, const uint32_t* ai, const int32_t* ao, uint64_t ant,
                                         const float* aes, const float* aee, const int32_t* aesrc, uint64_t ane,
                                         const float* bv, const uint32_t* bi, const int32_t* bo, uint64_t bnt,
                                         const float* bes, const float* bee, const int32_t* besrc, uint64_t bne,
                                         int direction, int max_iter, uint64_t* n_out) {
    Mesh A{av, ai, ao, ant}, B{bv, bi, bo, bnt};
    std::vector<uint64_t> keys;
    if (max_iter <= 0) max_iter = 100;  // the reference's default (mesh_overlap_edges.cu:111-112)
    if (direction == 0 || direction == 1) {
        Bvh bb;
        bb.build(B);
        edge_join_reference(aes, aee, aesrc, ane, B, bb, 0, max_iter, keys);
    }
    if (direction == 0 || direction == 2) {
        Bvh ab;
        ab.build(A);
        edge_join_reference(bes, bee, besrc, bne, A, ab, 1, max_iter, keys);
    }
    sort_unique(keys);
    return to_malloc(keys, n_out);
}

// Parity pairs of source first-vertices against target triangles; key is
// (src << 32 | tgt), or (tgt << 32 | src) when swap != 0.
uint64_t* oracle_parity_pairs(const float* first_vertices, int32_t nsrc, const float* tv, const uint32_t* ti,
                              const int32_t* to, uint64_t tnt, int swap, uint64_t* n_out) {
    Mesh T{tv, ti, to, tnt};
    Bvh bvh;
    bvh.build(T);
    std::vector<uint64_t> keys;
    parity_join(first_vertices, nsrc, T, bvh, swap, keys);
    sort_unique(keys);
    return to_malloc(keys, n_out);
}

// Parity-ray crossing counts: 2 * *n_out words, (src << 32 | tgt, count)
// per crossed (source, target) pair, in key order.
uint64_t* oracle_parity_crossings(const float* first_vertices, int32_t nsrc, const float* tv, const uint32_t* ti,
                                  const int32_t* to, uint64_t tnt, uint64_t* n_out) {
    Mesh T{tv, ti, to, tnt};
    Bvh bvh;
    bvh.build(T);
    std::vector<uint64_t> words;
    parity_crossings(first_vertices, nsrc, T, bvh, words);
    uint64_t n = 0;
    uint64_t* out = to_malloc(words, &n);
    *n_out = n / 2;
    return out;
}

// Face baseline restated: for every A triangle, every B triangle whose box
// meets it is tested with the exact closed triangle-triangle predicate (six
// exact edge-versus-triangle tests); OpenMP over A objects' triangles.  Only
// triangles [tri_begin, tri_end) of A are processed (bounded samples).
uint64_t* oracle_face_pairs(const float* av, const uint32_t* ai, const int32_t* ao, uint64_t ant,
                            const float* bv, const uint32_t* bi, const int32_t* bo, uint64_t bnt,
                            uint64_t tri_begin, uint64_t tri_end, uint64_t* n_out) {
    Mesh A{av, ai, ao, ant}, B{bv, bi, bo, bnt};
    Bvh bvh;
    bvh.build(B);
    if (tri_end > ant) tri_end = ant;
    int nth = 1;
#ifdef _OPENMP
    nth = omp_get_max_threads();
#endif
    std::vector<std::vector<uint64_t>> per(nth);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t t = (int64_t)tri_begin; t < (int64_t)tri_end; ++t) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        P3 a, b, c;
        A.tri((uint64_t)t, a, b, c);
        const Box tb = tri_box(a, b, c);
        const int32_t oa = A.obj[t];
        bvh.query([&](const Box& bx) { return boxes_overlap(tb, bx); },
                  [&](uint64_t u) {
                      P3 d, e, f;
                      B.tri(u, d, e, f);
                      const bool hit = seg_tri_exact(a, b, d, e, f) || seg_tri_exact(b, c, d, e, f) ||
                                       seg_tri_exact(c, a, d, e, f) || seg_tri_exact(d, e, a, b, c) ||
                                       seg_tri_exact(e, f, a, b, c) || seg_tri_exact(f, d, a, b, c);
                      if (hit) per[tid].push_back(pack(oa, B.obj[u]));
                  });
    }
    std::vector<uint64_t> keys;
    for (auto& v : per) keys.insert(keys.end(), v.begin(), v.end());
    sort_unique(keys);
    return to_malloc(keys, n_out);
}

// TOUCH baseline restated (baselines/face/src/touch_query.cpp): an STR tree
// of fanout 2 over A's object boxes (:125-219), B's objects assigned to it
// (:221-253), candidate pairs from the work nodes' descendant leaves
// (:268-302), then each candidate refined with the exact closed
// triangle-triangle predicate: any triangle of a against a hierarchy over
// b's triangles (:462-480, CGAL's do_intersect there).  Objects without
// triangles take no part.  OpenMP over the candidates.
uint64_t* oracle_touch_pairs(const float* av, const uint32_t* ai, const int32_t* ao, uint64_t ant,
                             const float* bv, const uint32_t* bi, const int32_t* bo, uint64_t bnt,
                             uint64_t* n_out, uint64_t* candidates_out) {
    Mesh A{av, ai, ao, ant}, B{bv, bi, bo, bnt};
    std::vector<uint64_t> keys;
    touch_join(A, B, keys, candidates_out);
    sort_unique(keys);
    return to_malloc(keys, n_out);
}

void oracle_free(void* p) { std::free(p); }

}  // extern "C"
