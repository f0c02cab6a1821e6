// Seeded synthetic dataset generators.
//
// The reference ships no datasets (its benchmarks download MICrONS meshes or
// instance template OBJ files), so the join workloads are generated here from
// a seed.  All arithmetic is IEEE basic operations in double precision with
// the deterministic series of detmath.h, rounded once to float32 per vertex
// coordinate, so a given seed yields bit-identical files on every host.
//
// Mesh families:
//  * icospheres: icosahedron subdivided `level` times, vertices projected to
//    the unit sphere (F = 20*4^level, V = 10*4^level + 2), scaled by a
//    lognormal radius and translated to a uniform centre;
//  * ellipsoids: the same template scaled per axis, rotated by a uniform
//    random rotation (Shoemake's quaternion method) and displaced radially by
//    smooth 3-D value noise;
//  * tubes: branching random-walk skeletons swept with an n-gon cross section
//    and closed with centre-fan caps.
// Every mesh is one object; object ids are dense 0..n-1 in generation order.
// Edges are extracted in per-object order (pierce::extract_edges order 1).
#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <utility>
#include <vector>

#include "detmath.h"
#include "geometry.h"
#include "icosphere.h"
#include "instance_math.h"

namespace {

using pierce::detm::Rng;

struct V3 {
    double x, y, z;
};
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 mul(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 normalize(V3 a) {
    double l = std::sqrt(dot(a, a));
    return l > 0 ? mul(a, 1.0 / l) : V3{0, 0, 1};
}

struct Template {
    std::vector<V3> verts;          // unit vectors
    std::vector<uint32_t> tris;     // 3 per triangle, outward CCW
};

Template make_icosphere(int level) {
    const pierce::inst::IcoTemplate h = pierce::inst::make_icosphere_template(level);
    Template t;
    for (size_t i = 0; i < h.v.size(); i += 3) t.verts.push_back({h.v[i], h.v[i + 1], h.v[i + 2]});
    t.tris = h.t;
    return t;
}

struct Rot {
    double m[9];
    V3 apply(V3 p) const {
        return {m[0] * p.x + m[1] * p.y + m[2] * p.z, m[3] * p.x + m[4] * p.y + m[5] * p.z,
                m[6] * p.x + m[7] * p.y + m[8] * p.z};
    }
};

// Uniform random rotation from three uniforms (Shoemake 1992).
Rot random_rotation(Rng& rng) {
    double u1 = rng.uniform(), u2 = rng.uniform(), u3 = rng.uniform();
    double s1 = std::sqrt(1.0 - u1), s2 = std::sqrt(u1);
    const double tp = pierce::detm::kTwoPi;
    double x = s1 * pierce::detm::sin(tp * u2), y = s1 * pierce::detm::cos(tp * u2);
    double z = s2 * pierce::detm::sin(tp * u3), w = s2 * pierce::detm::cos(tp * u3);
    Rot r;
    r.m[0] = 1 - 2 * (y * y + z * z);
    r.m[1] = 2 * (x * y - z * w);
    r.m[2] = 2 * (x * z + y * w);
    r.m[3] = 2 * (x * y + z * w);
    r.m[4] = 1 - 2 * (x * x + z * z);
    r.m[5] = 2 * (y * z - x * w);
    r.m[6] = 2 * (x * z - y * w);
    r.m[7] = 2 * (y * z + x * w);
    r.m[8] = 1 - 2 * (x * x + y * y);
    return r;
}

struct EllipsoidParams {
    V3 center;
    double ax, ay, az;
    Rot rot;
    uint64_t noise_seed;
    V3 noise_offset;
};

EllipsoidParams random_ellipsoid(Rng& rng, double lo, double hi, double axis_lo, double axis_hi) {
    EllipsoidParams p;
    p.center.x = rng.uniform(lo, hi);
    p.center.y = rng.uniform(lo, hi);
    p.center.z = rng.uniform(lo, hi);
    p.ax = rng.uniform(axis_lo, axis_hi);
    p.ay = rng.uniform(axis_lo, axis_hi);
    p.az = rng.uniform(axis_lo, axis_hi);
    p.rot = random_rotation(rng);
    p.noise_seed = rng.next();
    p.noise_offset = {rng.uniform(0, 64), rng.uniform(0, 64), rng.uniform(0, 64)};
    return p;
}

// Append one mesh (template topology, given vertex positions) as object `obj`.
void append_mesh(pierce_geom& g, const Template& t, const std::vector<float>& pos, int32_t obj) {
    const uint32_t base = (uint32_t)g.num_vertices();
    g.vertices.insert(g.vertices.end(), pos.begin(), pos.end());
    for (size_t i = 0; i < t.tris.size(); ++i) g.indices.push_back(base + t.tris[i]);
    g.tri_to_object.insert(g.tri_to_object.end(), t.tris.size() / 3, obj);
}

pierce_mesh_instance to_instance(const EllipsoidParams& p, double noise_amp, int level) {
    pierce_mesh_instance m{};
    m.center[0] = p.center.x;
    m.center[1] = p.center.y;
    m.center[2] = p.center.z;
    m.axes[0] = p.ax;
    m.axes[1] = p.ay;
    m.axes[2] = p.az;
    for (int k = 0; k < 9; ++k) m.rotation[k] = p.rot.m[k];
    m.noise_amp = noise_amp;
    m.noise_offset[0] = p.noise_offset.x;
    m.noise_offset[1] = p.noise_offset.y;
    m.noise_offset[2] = p.noise_offset.z;
    m.noise_seed = p.noise_seed;
    m.level = level;
    return m;
}

void instance_positions(const Template& t, const pierce_mesh_instance& m, std::vector<float>& out) {
    out.resize(3 * t.verts.size());
    for (size_t i = 0; i < t.verts.size(); ++i)
        pierce::inst::instance_vertex(m, t.verts[i].x, t.verts[i].y, t.verts[i].z, &out[3 * i]);
}

void ellipsoid_positions(const Template& t, const EllipsoidParams& p, double noise_amp, std::vector<float>& out) {
    instance_positions(t, to_instance(p, noise_amp, 0), out);
}

void finish(pierce_geom& g) {
    g.total_triangles = g.num_triangles();
    pierce::extract_edges(g, 1, 0);
}

// ---- tubes ---------------------------------------------------------------

V3 random_unit(Rng& rng) {
    // Uniform direction from a normal triple.
    for (;;) {
        V3 v{rng.normal(), rng.normal(), rng.normal()};
        double l2 = dot(v, v);
        if (l2 > 1e-12) return mul(v, 1.0 / std::sqrt(l2));
    }
}

// Sweep an n-gon along a polyline and cap both ends with centre fans:
// m*n ring vertices then the two cap centres; per segment and side two
// triangles (a, b, d), (a, d, c); then the first cap's fan, then the last's.  The
// unique edges are listed structurally, each once: the ring edges of every
// ring, the longitudinal and the diagonal edge of every segment side, and
// the spokes of both caps (3 m n edges for m rings).
struct Branch {
    std::vector<V3> pts;
    double radius;
    int32_t obj;
};

inline int64_t branch_vertices(const Branch& b, int n) { return b.pts.size() < 2 ? 0 : (int64_t)b.pts.size() * n + 2; }
inline int64_t branch_triangles(const Branch& b, int n) {
    return b.pts.size() < 2 ? 0 : 2 * (int64_t)n * ((int64_t)b.pts.size() - 1) + 2 * (int64_t)n;
}
inline int64_t branch_edges(const Branch& b, int n) { return b.pts.size() < 2 ? 0 : 3 * (int64_t)b.pts.size() * n; }

void sweep_branch(const Branch& br, int n, uint32_t base, float* vout, uint32_t* iout, int32_t* tout, float* es,
                  float* ee, int32_t* esrc) {
    const std::vector<V3>& pts = br.pts;
    if (pts.size() < 2) return;
    const double radius = br.radius;
    // Frames by parallel transport of an initial perpendicular.
    V3 t0 = normalize(sub(pts[1], pts[0]));
    V3 helper = std::fabs(t0.z) < 0.9 ? V3{0, 0, 1} : V3{1, 0, 0};
    V3 u = normalize(cross(t0, helper));
    const size_t m = pts.size();
    float* v = vout;
    for (size_t i = 0; i < m; ++i) {
        V3 ti = (i + 1 < m) ? sub(pts[i + 1], pts[i]) : sub(pts[i], pts[i - 1]);
        if (i > 0 && i + 1 < m) ti = add(normalize(sub(pts[i + 1], pts[i])), normalize(sub(pts[i], pts[i - 1])));
        ti = normalize(ti);
        u = normalize(sub(u, mul(ti, dot(u, ti))));
        V3 w = cross(ti, u);
        for (int k = 0; k < n; ++k) {
            double ang = pierce::detm::kTwoPi * (double)k / (double)n;
            V3 q = add(pts[i], add(mul(u, radius * pierce::detm::cos(ang)), mul(w, radius * pierce::detm::sin(ang))));
            *v++ = (float)q.x;
            *v++ = (float)q.y;
            *v++ = (float)q.z;
        }
    }
    *v++ = (float)pts[0].x;
    *v++ = (float)pts[0].y;
    *v++ = (float)pts[0].z;
    *v++ = (float)pts[m - 1].x;
    *v++ = (float)pts[m - 1].y;
    *v++ = (float)pts[m - 1].z;
    const uint32_t c0 = base + (uint32_t)(m * n), c1 = c0 + 1;
    uint32_t* ix = iout;
    for (size_t i = 0; i + 1 < m; ++i) {
        for (int k = 0; k < n; ++k) {
            uint32_t a = base + (uint32_t)(i * n + k), b = base + (uint32_t)(i * n + (k + 1) % n);
            uint32_t c = a + (uint32_t)n, d = b + (uint32_t)n;
            const uint32_t q[6] = {a, b, d, a, d, c};
            ix = std::copy(q, q + 6, ix);
        }
    }
    // each cap's fan in one run, so consecutive triangles stay close together
    for (int k = 0; k < n; ++k) {
        uint32_t a = base + (uint32_t)k, b = base + (uint32_t)((k + 1) % n);
        const uint32_t f0[3] = {c0, b, a};
        ix = std::copy(f0, f0 + 3, ix);
    }
    for (int k = 0; k < n; ++k) {
        uint32_t la = base + (uint32_t)((m - 1) * n + k), lb = base + (uint32_t)((m - 1) * n + (k + 1) % n);
        const uint32_t f1[3] = {c1, la, lb};
        ix = std::copy(f1, f1 + 3, ix);
    }
    std::fill(tout, tout + branch_triangles(br, n), br.obj);
    // structural unique edges (vertex indices local to the branch)
    auto vert = [&](uint32_t local) { return vout + 3 * (size_t)local; };
    size_t e = 0;
    auto emit = [&](uint32_t la, uint32_t lb) {
        std::copy(vert(la), vert(la) + 3, es + 3 * e);
        std::copy(vert(lb), vert(lb) + 3, ee + 3 * e);
        esrc[e] = br.obj;
        ++e;
    };
    for (size_t i = 0; i < m; ++i)
        for (int k = 0; k < n; ++k) {
            const uint32_t a = (uint32_t)(i * n + k), b = (uint32_t)(i * n + (k + 1) % n);
            emit(a, b);  // ring edge
            if (i + 1 < m) {
                emit(a, a + (uint32_t)n);  // longitudinal
                emit(a, b + (uint32_t)n);  // diagonal
            }
        }
    for (int k = 0; k < n; ++k) {
        emit((uint32_t)(m * n), (uint32_t)k);                            // first cap spoke
        emit((uint32_t)(m * n + 1), (uint32_t)((m - 1) * n + k));        // last cap spoke
    }
}

}  // namespace

// Unit icosphere template of one subdivision level: vertices (double xyz),
// triangles and the unique undirected edges (each once, first-seen
// orientation, in first-seen order).  Used to expand instanced datasets on
// the device.
extern "C" int pierce_icosphere_template(int32_t level, double* vertices, uint32_t* tris, uint32_t* edges,
                                         int64_t* counts) {
    if (level < 0 || level > 8 || !counts) {
        pierce::set_last_error("icosphere_template: invalid argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    const pierce::inst::IcoTemplate h = pierce::inst::make_icosphere_template(level);
    Template t = make_icosphere(level);
    const std::vector<uint32_t>& e = h.e;
    counts[0] = (int64_t)t.verts.size();
    counts[1] = (int64_t)(t.tris.size() / 3);
    counts[2] = (int64_t)(e.size() / 2);
    if (vertices)
        for (size_t i = 0; i < t.verts.size(); ++i) {
            vertices[3 * i] = t.verts[i].x;
            vertices[3 * i + 1] = t.verts[i].y;
            vertices[3 * i + 2] = t.verts[i].z;
        }
    if (tris) std::copy(t.tris.begin(), t.tris.end(), tris);
    if (edges) std::copy(e.begin(), e.end(), edges);
    return PIERCE_HOST_OK;
}

extern "C" int pierce_gen_icospheres(uint64_t seed, int32_t num_meshes, int32_t level, double ln_mu, double sigma,
                                     double lo, double hi, pierce_geom** out) {
    if (!out || num_meshes < 0 || level < 0 || level > 8) {
        pierce::set_last_error("gen_icospheres: invalid argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    Template t = make_icosphere(level);
    std::unique_ptr<pierce_geom> g(new pierce_geom());
    g->vertices.reserve((size_t)num_meshes * 3 * t.verts.size());
    g->indices.reserve((size_t)num_meshes * t.tris.size());
    Rng rng(seed);
    std::vector<float> pos(3 * t.verts.size());
    for (int32_t m = 0; m < num_meshes; ++m) {
        V3 c{rng.uniform(lo, hi), rng.uniform(lo, hi), rng.uniform(lo, hi)};
        double r = pierce::detm::exp(ln_mu + sigma * rng.normal());
        for (size_t i = 0; i < t.verts.size(); ++i) {
            pos[3 * i + 0] = (float)(c.x + r * t.verts[i].x);
            pos[3 * i + 1] = (float)(c.y + r * t.verts[i].y);
            pos[3 * i + 2] = (float)(c.z + r * t.verts[i].z);
        }
        append_mesh(*g, t, pos, m);
    }
    finish(*g);
    *out = g.release();
    return PIERCE_HOST_OK;
}

extern "C" int pierce_gen_ellipsoid_pair(uint64_t seed_a, uint64_t seed_b, int32_t num_a, int32_t num_b,
                                         int32_t level, double axis_lo, double axis_hi, double noise_amp, double lo,
                                         double hi, double frac_inside, double inside_scale, double frac_contact,
                                         pierce_geom** out_a, pierce_geom** out_b) {
    if (!out_a || !out_b || num_a < 0 || num_b < 0 || level < 0 || level > 8 ||
        ((frac_inside > 0 || frac_contact > 0) && num_a == 0)) {
        pierce::set_last_error("gen_ellipsoid_pair: invalid argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    Template t = make_icosphere(level);
    std::unique_ptr<pierce_geom> A(new pierce_geom()), B(new pierce_geom());
    const size_t nvm = t.verts.size();
    A->vertices.reserve((size_t)num_a * 3 * nvm);
    B->vertices.reserve((size_t)num_b * 3 * nvm);
    std::vector<EllipsoidParams> params_a((size_t)num_a);
    Rng ra(seed_a);
    std::vector<float> pos;
    for (int32_t m = 0; m < num_a; ++m) {
        params_a[m] = random_ellipsoid(ra, lo, hi, axis_lo, axis_hi);
        ellipsoid_positions(t, params_a[m], noise_amp, pos);
        append_mesh(*A, t, pos, m);
    }
    Rng rb(seed_b);
    for (int32_t m = 0; m < num_b; ++m) {
        const double u = rb.uniform();
        EllipsoidParams own = random_ellipsoid(rb, lo, hi, axis_lo, axis_hi);
        if (u < frac_inside) {
            // Scaled copy of a random A mesh about its generation centre: the
            // meshes are star-shaped about that centre, so the copy is inside.
            const int32_t j = (int32_t)rb.below((uint64_t)num_a);
            const EllipsoidParams& pa = params_a[j];
            pos.resize(3 * nvm);
            const float* va = &A->vertices[(size_t)j * 3 * nvm];
            for (size_t i = 0; i < nvm; ++i) {
                pos[3 * i + 0] = (float)(pa.center.x + inside_scale * ((double)va[3 * i + 0] - pa.center.x));
                pos[3 * i + 1] = (float)(pa.center.y + inside_scale * ((double)va[3 * i + 1] - pa.center.y));
                pos[3 * i + 2] = (float)(pa.center.z + inside_scale * ((double)va[3 * i + 2] - pa.center.z));
            }
        } else if (u < frac_inside + frac_contact) {
            const int32_t j = (int32_t)rb.below((uint64_t)num_a);
            const float* va = &A->vertices[(size_t)j * 3 * nvm];
            if (rb.uniform() < 0.5) {
                // Exact duplicate of A_j: every face coplanar with a face of A_j.
                pos.assign(va, va + 3 * nvm);
            } else {
                // Own ellipsoid resting on A_j: its lowest vertex is moved onto
                // A_j's highest vertex exactly (a single-point contact).
                ellipsoid_positions(t, own, noise_amp, pos);
                size_t kb = 0, ka = 0;
                for (size_t i = 1; i < nvm; ++i) {
                    if (pos[3 * i + 2] < pos[3 * kb + 2]) kb = i;
                    if (va[3 * i + 2] > va[3 * ka + 2]) ka = i;
                }
                const double tx = (double)va[3 * ka + 0] - (double)pos[3 * kb + 0];
                const double ty = (double)va[3 * ka + 1] - (double)pos[3 * kb + 1];
                const double tz = (double)va[3 * ka + 2] - (double)pos[3 * kb + 2];
                for (size_t i = 0; i < nvm; ++i) {
                    pos[3 * i + 0] = (float)((double)pos[3 * i + 0] + tx);
                    pos[3 * i + 1] = (float)((double)pos[3 * i + 1] + ty);
                    pos[3 * i + 2] = (float)((double)pos[3 * i + 2] + tz);
                }
                pos[3 * kb + 0] = va[3 * ka + 0];
                pos[3 * kb + 1] = va[3 * ka + 1];
                pos[3 * kb + 2] = va[3 * ka + 2];
            }
        } else {
            ellipsoid_positions(t, own, noise_amp, pos);
        }
        append_mesh(*B, t, pos, m);
    }
    finish(*A);
    finish(*B);
    *out_a = A.release();
    *out_b = B.release();
    return PIERCE_HOST_OK;
}

namespace {

// Tubes 0 .. num_meshes - 1 from one random stream; only the branches of
// meshes below `sweep_meshes` are swept into the output.
int gen_tubes(uint64_t seed, int32_t num_meshes, int32_t sweep_meshes, int64_t target_tris, double step,
              double branch_prob, double r_lo, double r_hi, int32_t n_sides, double lo, double hi, pierce_geom** out) {
    if (!out || num_meshes < 0 || target_tris <= 0 || n_sides < 3 || step <= 0) {
        pierce::set_last_error("gen_tubes: invalid argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    // 1. skeletons, one random stream in mesh order
    std::vector<Branch> branches;
    Rng rng(seed);
    const int64_t tris_per_segment = 2 * (int64_t)n_sides;
    for (int32_t m = 0; m < num_meshes; ++m) {
        const double radius = rng.uniform(r_lo, r_hi);
        struct Start {
            V3 p, d;
        };
        std::vector<Start> pending;
        pending.push_back({{rng.uniform(lo, hi), rng.uniform(lo, hi), rng.uniform(lo, hi)}, random_unit(rng)});
        int64_t budget = target_tris;
        while (!pending.empty() && budget > 2 * n_sides + tris_per_segment) {
            Start s = pending.back();
            pending.pop_back();
            Branch br{{s.p}, radius, m};
            V3 p = s.p, d = s.d;
            budget -= 2 * n_sides;  // caps
            while (budget >= tris_per_segment) {
                d = normalize(add(d, mul(random_unit(rng), 0.35)));
                p = add(p, mul(d, step));
                br.pts.push_back(p);
                budget -= tris_per_segment;
                if (rng.uniform() < branch_prob) pending.push_back({p, normalize(add(d, random_unit(rng)))});
                // Branches end with probability 1/400 per segment once a
                // branch is queued, so the budget spreads over several arms.
                if (!pending.empty() && rng.uniform() < 1.0 / 400.0) break;
            }
            if (br.pts.size() >= 2 && m < sweep_meshes) branches.push_back(std::move(br));
        }
    }
    // 2. offsets, then every branch swept in parallel into its own ranges
    const size_t nb = branches.size();
    std::vector<int64_t> vo(nb + 1, 0), to(nb + 1, 0), eo(nb + 1, 0);
    for (size_t i = 0; i < nb; ++i) {
        vo[i + 1] = vo[i] + branch_vertices(branches[i], n_sides);
        to[i + 1] = to[i] + branch_triangles(branches[i], n_sides);
        eo[i + 1] = eo[i] + branch_edges(branches[i], n_sides);
    }
    if (vo[nb] >= (int64_t)1 << 32) {
        pierce::set_last_error("gen_tubes: more than 2^32 vertices");
        return PIERCE_HOST_ERR_INVALID;
    }
    std::unique_ptr<pierce_geom> g(new pierce_geom());
    g->vertices.resize(3 * (size_t)vo[nb]);
    g->indices.resize(3 * (size_t)to[nb]);
    g->tri_to_object.resize((size_t)to[nb]);
    g->edge_starts.resize(3 * (size_t)eo[nb]);
    g->edge_ends.resize(3 * (size_t)eo[nb]);
    g->edge_src.resize((size_t)eo[nb]);
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t i = 0; i < (int64_t)nb; ++i)
        sweep_branch(branches[i], n_sides, (uint32_t)vo[i], &g->vertices[3 * vo[i]], &g->indices[3 * to[i]],
                     &g->tri_to_object[to[i]], &g->edge_starts[3 * eo[i]], &g->edge_ends[3 * eo[i]],
                     &g->edge_src[eo[i]]);
    g->total_triangles = g->num_triangles();
    *out = g.release();
    return PIERCE_HOST_OK;
}

}  // namespace

extern "C" int pierce_gen_tubes(uint64_t seed, int32_t num_meshes, int64_t target_tris, double step,
                                double branch_prob, double r_lo, double r_hi, int32_t n_sides, double lo, double hi,
                                pierce_geom** out) {
    return gen_tubes(seed, num_meshes, num_meshes, target_tris, step, branch_prob, r_lo, r_hi, n_sides, lo, hi, out);
}

extern "C" int pierce_gen_tubes_head(uint64_t seed, int32_t num_meshes, int32_t first_meshes, int64_t target_tris,
                                     double step, double branch_prob, double r_lo, double r_hi, int32_t n_sides,
                                     double lo, double hi, pierce_geom** out) {
    if (first_meshes < 0 || first_meshes > num_meshes) {
        pierce::set_last_error("gen_tubes_head: first_meshes out of range");
        return PIERCE_HOST_ERR_INVALID;
    }
    return gen_tubes(seed, num_meshes, first_meshes, target_tris, step, branch_prob, r_lo, r_hi, n_sides, lo, hi, out);
}

// ---- instanced icosphere datasets -------------------------------------------

extern "C" int pierce_gen_instances(uint64_t seed, int32_t num_meshes, int32_t family, int32_t level_lo,
                                    int32_t level_hi, double p0, double p1, double noise_amp, double lo, double hi,
                                    pierce_mesh_instance* out) {
    if ((!out && num_meshes) || num_meshes < 0 || (family != 0 && family != 1) || level_lo < 0 ||
        level_hi < level_lo || level_hi > PIERCE_MAX_INSTANCE_LEVEL) {
        pierce::set_last_error("gen_instances: invalid argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    Rng rng(seed);
    for (int32_t m = 0; m < num_meshes; ++m) {
        pierce_mesh_instance& r = out[m];
        if (family == 0) {
            r = pierce_mesh_instance{};
            r.center[0] = rng.uniform(lo, hi);
            r.center[1] = rng.uniform(lo, hi);
            r.center[2] = rng.uniform(lo, hi);
            const double radius = pierce::detm::exp(p0 + p1 * rng.normal());
            r.axes[0] = r.axes[1] = r.axes[2] = radius;
            r.rotation[0] = r.rotation[4] = r.rotation[8] = 1.0;
        } else {
            r = to_instance(random_ellipsoid(rng, lo, hi, p0, p1), noise_amp, 0);
        }
        r.level = level_lo == level_hi ? level_lo : level_lo + (int32_t)rng.below((uint64_t)(level_hi - level_lo + 1));
    }
    return PIERCE_HOST_OK;
}

extern "C" int pierce_expand_instances(const pierce_mesh_instance* meshes, int32_t num_meshes, pierce_geom** out) {
    if (!out || (!meshes && num_meshes) || num_meshes < 0) {
        pierce::set_last_error("expand_instances: invalid argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    for (int32_t m = 0; m < num_meshes; ++m)
        if (meshes[m].level < 0 || meshes[m].level > PIERCE_MAX_INSTANCE_LEVEL) {
            pierce::set_last_error("expand_instances: level out of range");
            return PIERCE_HOST_ERR_INVALID;
        }
    std::map<int, std::pair<Template, std::vector<uint32_t>>> templates;
    std::unique_ptr<pierce_geom> g(new pierce_geom());
    std::vector<float> pos;
    for (int32_t m = 0; m < num_meshes; ++m) {
        auto it = templates.find(meshes[m].level);
        if (it == templates.end()) {
            Template t = make_icosphere(meshes[m].level);
            std::vector<uint32_t> e = pierce::inst::make_icosphere_template(meshes[m].level).e;
            it = templates.emplace(meshes[m].level, std::make_pair(std::move(t), std::move(e))).first;
        }
        const Template& t = it->second.first;
        const std::vector<uint32_t>& e = it->second.second;
        instance_positions(t, meshes[m], pos);
        append_mesh(*g, t, pos, m);
        for (size_t k = 0; k < e.size(); k += 2) {
            g->edge_starts.insert(g->edge_starts.end(), &pos[3 * e[k]], &pos[3 * e[k]] + 3);
            g->edge_ends.insert(g->edge_ends.end(), &pos[3 * e[k + 1]], &pos[3 * e[k + 1]] + 3);
            g->edge_src.push_back(m);
        }
    }
    g->total_triangles = g->num_triangles();
    *out = g.release();
    return PIERCE_HOST_OK;
}
