// Unique-edge extraction and grid statistics for the `.pre` producer.
//
// Edge semantics follow EdgePreprocessor::extractEdges
// (pierce/preprocess/src/EdgePreprocessor.cpp:44-111):
//  * every triangle (in index order) contributes its three directed edges
//    v0->v1, v1->v2, v2->v0; triangles with an out-of-range vertex index are
//    skipped, and nothing is produced when triangleToObject and the index
//    array differ in length;
//  * endpoints are quantised to int64 with llround(double(x) * 1e5);
//  * the key is (min(q0,q1), max(q0,q1), objectId) with points compared
//    lexicographically; the first triangle edge that produces a key wins and
//    keeps its own (unswapped) float endpoints;
//  * output order is ascending key order (the std::map iteration order).
// Here the map is replaced, per object and in parallel, by a hash set that
// keeps the first arrival of each key (records are generated in arrival
// order) and a sort of the surviving records by key: equal keys always
// share an object, so "first arrival per key" is decided inside one object.  order == 0 then merges all
// objects into global key order (byte-identical to the reference output);
// order == 1 keeps objects in id order (same edge set, cheaper for large
// datasets whose edge order does not matter to the join).
//
// Grid statistics follow generateGridStats
// (pierce/preprocess/src/pierce_preprocess.cpp:49-167).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <numeric>
#include <tuple>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#include <parallel/algorithm>
#endif

#include "geometry.h"

namespace {

struct EdgeRec {
    int64_t a[3];
    int64_t b[3];
    int32_t obj;
    uint32_t corner;  // 0..2: which edge of the triangle
    uint64_t tri;     // triangle index (arrival order = tri*3 + corner)
};

inline bool key_less(const EdgeRec& x, const EdgeRec& y) {
    for (int i = 0; i < 3; ++i)
        if (x.a[i] != y.a[i]) return x.a[i] < y.a[i];
    for (int i = 0; i < 3; ++i)
        if (x.b[i] != y.b[i]) return x.b[i] < y.b[i];
    return x.obj < y.obj;
}
inline bool key_equal(const EdgeRec& x, const EdgeRec& y) {
    return x.obj == y.obj && std::memcmp(x.a, y.a, sizeof(x.a)) == 0 &&
           std::memcmp(x.b, y.b, sizeof(x.b)) == 0;
}
// Hash of a record's key (both quantised endpoints and the object id),
// 64-bit multiply-xorshift mixing.
inline uint64_t key_hash(const EdgeRec& r) {
    uint64_t h = 0x9E3779B97F4A7C15ull ^ (uint64_t)(uint32_t)r.obj;
    for (int i = 0; i < 3; ++i) {
        h = (h ^ (uint64_t)r.a[i]) * 0xff51afd7ed558ccdull;
        h ^= h >> 33;
    }
    for (int i = 0; i < 3; ++i) {
        h = (h ^ (uint64_t)r.b[i]) * 0xc4ceb9fe1a85ec53ull;
        h ^= h >> 33;
    }
    return h;
}

// llround(double(x) * 1e5) without the libm call: truncate, then round half
// away from zero on the exact remainder (x - trunc(x) is exact below 2^52).
inline int64_t round_half_away(double x) {
    if (!(std::fabs(x) < 4.0e18)) return (int64_t)std::llround(x);
    int64_t i = (int64_t)x;
    double frac = x - (double)i;
    if (frac >= 0.5) ++i;
    else if (frac <= -0.5) --i;
    return i;
}

inline void quantise(const float* p, int64_t q[3]) {
    for (int i = 0; i < 3; ++i) q[i] = round_half_away((double)p[i] * 1e5);
}

inline bool point_less(const int64_t* x, const int64_t* y) {
    if (x[0] != y[0]) return x[0] < y[0];
    if (x[1] != y[1]) return x[1] < y[1];
    return x[2] < y[2];
}

}  // namespace

namespace pierce {

void extract_edges(pierce_geom& g, int order, int num_threads) {
    g.edge_starts.clear();
    g.edge_ends.clear();
    g.edge_src.clear();
    const uint64_t nt = g.num_triangles();
    const uint64_t nv = g.num_vertices();
    if (nt == 0 || nv == 0 || g.tri_to_object.size() != nt) return;

    // Thread count of this call only (the process-wide OpenMP setting stays
    // as it is): num_threads > 0, else every thread OpenMP offers.
    int nthreads = 1;
#ifdef _OPENMP
    nthreads = num_threads > 0 ? num_threads : omp_get_max_threads();
#else
    (void)num_threads;
#endif

    // Group triangles by object id with a counting sort (objects may have
    // negative ids in hostile inputs; those are grouped separately at the end).
    int32_t max_obj = -1;
    for (int32_t o : g.tri_to_object) max_obj = std::max(max_obj, o);
    const int64_t nobj = (int64_t)max_obj + 2;  // last bucket: negative ids
    std::vector<uint64_t> start(nobj + 1, 0);
    auto bucket = [&](int32_t o) -> int64_t { return o < 0 ? nobj - 1 : (int64_t)o; };
    for (uint64_t t = 0; t < nt; ++t) start[bucket(g.tri_to_object[t]) + 1]++;
    for (int64_t i = 0; i < nobj; ++i) start[i + 1] += start[i];
    std::vector<uint64_t> tris(nt);
    {
        std::vector<uint64_t> cur(start.begin(), start.end() - 1);
        for (uint64_t t = 0; t < nt; ++t) tris[cur[bucket(g.tri_to_object[t])]++] = t;
    }

    // Per-object unique edges, each object's list in key order.  Each thread
    // sorts one object's records in a reused buffer and appends the survivors
    // (triangle, corner) to its own arena; objects are then laid out in id
    // order.  Memory stays O(largest object) per thread plus the output.
    struct Ref {
        uint64_t tri;
        uint32_t corner;
        int32_t obj;
    };
    struct Slot {
        int arena;
        uint64_t offset, count;
    };
    std::vector<std::vector<Ref>> arenas(nthreads);
    std::vector<Slot> slots(nobj);
#pragma omp parallel num_threads(nthreads)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        std::vector<EdgeRec> buf, uniq;
        std::vector<size_t> table;
        std::vector<Ref>& arena = arenas[tid];
#pragma omp for schedule(dynamic, 16)
        for (int64_t o = 0; o < nobj; ++o) {
            buf.clear();
            for (uint64_t k = start[o]; k < start[o + 1]; ++k) {
                const uint64_t t = tris[k];
                const uint32_t* tri = &g.indices[3 * t];
                if (tri[0] >= nv || tri[1] >= nv || tri[2] >= nv) continue;
                int64_t q[3][3];
                for (int c = 0; c < 3; ++c) quantise(&g.vertices[3 * (uint64_t)tri[c]], q[c]);
                for (uint32_t e = 0; e < 3; ++e) {
                    EdgeRec r;
                    const int64_t* q0 = q[e];
                    const int64_t* q1 = q[(e + 1) % 3];
                    if (point_less(q1, q0)) std::swap(q0, q1);
                    std::memcpy(r.a, q0, sizeof(r.a));
                    std::memcpy(r.b, q1, sizeof(r.b));
                    r.obj = g.tri_to_object[t];
                    r.corner = e;
                    r.tri = t;
                    buf.push_back(r);
                }
            }
            // records are in arrival order (triangles ascending, then
            // corners): the first insert of a key is its first arrival
            size_t cap = 16;
            while (cap < 2 * buf.size()) cap <<= 1;
            table.assign(cap, SIZE_MAX);
            uniq.clear();
            for (const EdgeRec& r : buf) {
                size_t h = (size_t)key_hash(r) & (cap - 1);
                for (;;) {
                    const size_t j = table[h];
                    if (j == SIZE_MAX) {
                        table[h] = uniq.size();
                        uniq.push_back(r);
                        break;
                    }
                    if (key_equal(uniq[j], r)) break;
                    h = (h + 1) & (cap - 1);
                }
            }
            std::sort(uniq.begin(), uniq.end(), key_less);  // keys are unique here
            Slot s{tid, arena.size(), uniq.size()};
            for (const EdgeRec& r : uniq) arena.push_back(Ref{r.tri, r.corner, r.obj});
            slots[o] = s;
        }
    }
    std::vector<uint64_t> off(nobj + 1, 0);
    for (int64_t o = 0; o < nobj; ++o) off[o + 1] = off[o] + slots[o].count;
    const uint64_t ne = off[nobj];
    std::vector<Ref> all(ne);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (int64_t o = 0; o < nobj; ++o) {
        const Slot& s = slots[o];
        if (s.count)
            std::memcpy(&all[off[o]], &arenas[s.arena][s.offset], s.count * sizeof(Ref));
    }
    arenas.clear();

    if (order == 0) {
        // Global key order: rebuild keys for the unique edges and sort them.
        // uninitialised storage: every record is written below
        std::unique_ptr<EdgeRec[]> keyed(new EdgeRec[ne]);
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (int64_t i = 0; i < (int64_t)ne; ++i) {
            const Ref& r = all[i];
            const uint32_t* tri = &g.indices[3 * r.tri];
            int64_t q0[3], q1[3];
            quantise(&g.vertices[3 * (uint64_t)tri[r.corner]], q0);
            quantise(&g.vertices[3 * (uint64_t)tri[(r.corner + 1) % 3]], q1);
            const int64_t* lo = q0;
            const int64_t* hi = q1;
            if (point_less(q1, q0)) std::swap(lo, hi);
            EdgeRec& k = keyed[i];
            std::memcpy(k.a, lo, sizeof(k.a));
            std::memcpy(k.b, hi, sizeof(k.b));
            k.obj = r.obj;
            k.corner = r.corner;
            k.tri = r.tri;
        }
        // Each object's records form a run sorted by key (the runs lie in
        // object order): a multiway merge of the runs gives the global order.
#ifdef _OPENMP
        std::vector<std::pair<EdgeRec*, EdgeRec*>> runs;
        runs.reserve((size_t)nobj);
        for (int64_t o = 0; o < nobj; ++o)
            if (off[o + 1] > off[o]) runs.emplace_back(keyed.get() + off[o], keyed.get() + off[o + 1]);
        std::unique_ptr<EdgeRec[]> merged(new EdgeRec[ne]);
        __gnu_parallel::multiway_merge(runs.begin(), runs.end(), merged.get(), (int64_t)ne, key_less,
                                       __gnu_parallel::default_parallel_tag((__gnu_parallel::_ThreadIndex)nthreads));
        keyed.swap(merged);
#else
        std::sort(keyed.get(), keyed.get() + ne, key_less);
#endif
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (int64_t i = 0; i < (int64_t)ne; ++i) all[i] = Ref{keyed[i].tri, keyed[i].corner, keyed[i].obj};
    }

    g.edge_starts.resize(3 * ne);
    g.edge_ends.resize(3 * ne);
    g.edge_src.resize(ne);
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t i = 0; i < (int64_t)ne; ++i) {
        const Ref& r = all[i];
        const uint32_t* tri = &g.indices[3 * r.tri];
        const float* p0 = &g.vertices[3 * (uint64_t)tri[r.corner]];
        const float* p1 = &g.vertices[3 * (uint64_t)tri[(r.corner + 1) % 3]];
        std::memcpy(&g.edge_starts[3 * i], p0, 3 * sizeof(float));
        std::memcpy(&g.edge_ends[3 * i], p1, 3 * sizeof(float));
        g.edge_src[i] = r.obj;
    }
}

void grid_stats(pierce_geom& g, float cell_size) {
    // Objects run in parallel; every floating-point sum keeps the order of
    // a serial pass (an object's triangles ascending, a cell's objects
    // ascending), so the statistics do not depend on the thread count.
    struct ObjStats {
        float mn[3] = {1e30f, 1e30f, 1e30f};
        float mx[3] = {-1e30f, -1e30f, -1e30f};
        double volume = 0.0;
        bool seen = false;
    };
    const uint64_t nt = g.num_triangles(), nv = g.num_vertices();
    const uint64_t nmap = std::min<uint64_t>(nt, g.tri_to_object.size());
    int32_t max_obj = -1;
    for (uint64_t t = 0; t < nmap; ++t) max_obj = std::max(max_obj, g.tri_to_object[t]);
    const int64_t nobj = (int64_t)max_obj + 1;
    std::vector<ObjStats> objs((size_t)nobj);
    auto valid = [&](uint64_t t) {
        const uint32_t* tri = &g.indices[3 * t];
        return g.tri_to_object[t] >= 0 && tri[0] < nv && tri[1] < nv && tri[2] < nv;
    };
    // triangles grouped by object, ascending within each object
    std::vector<uint64_t> start((size_t)nobj + 1, 0);
    for (uint64_t t = 0; t < nmap; ++t)
        if (valid(t)) start[(size_t)g.tri_to_object[t] + 1]++;
    for (int64_t o = 0; o < nobj; ++o) start[o + 1] += start[o];
    std::vector<uint64_t> tris(start[(size_t)nobj]);
    {
        std::vector<uint64_t> cur(start.begin(), start.end() - 1);
        for (uint64_t t = 0; t < nmap; ++t)
            if (valid(t)) tris[cur[(size_t)g.tri_to_object[t]]++] = t;
    }
    // Per object: bounding box, then the signed volume relative to the box
    // centre (float products summed in double as in the reference).
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t o = 0; o < nobj; ++o) {
        ObjStats& s = objs[o];
        for (uint64_t k = start[o]; k < start[o + 1]; ++k) {
            const uint32_t* tri = &g.indices[3 * tris[k]];
            s.seen = true;
            for (int j = 0; j < 3; ++j) {
                const float* v = &g.vertices[3 * (uint64_t)tri[j]];
                for (int d = 0; d < 3; ++d) {
                    s.mn[d] = std::min(s.mn[d], v[d]);
                    s.mx[d] = std::max(s.mx[d], v[d]);
                }
            }
        }
        float c[3];
        for (int d = 0; d < 3; ++d) c[d] = (s.mn[d] + s.mx[d]) * 0.5f;
        for (uint64_t k = start[o]; k < start[o + 1]; ++k) {
            const uint32_t* tri = &g.indices[3 * tris[k]];
            float p[3][3];
            for (int j = 0; j < 3; ++j)
                for (int d = 0; d < 3; ++d) p[j][d] = g.vertices[3 * (uint64_t)tri[j] + d] - c[d];
            float cx = p[0][1] * p[1][2] - p[0][2] * p[1][1];
            float cy = p[0][2] * p[1][0] - p[0][0] * p[1][2];
            float cz = p[0][0] * p[1][1] - p[0][1] * p[1][0];
            s.volume += (cx * p[2][0] + cy * p[2][1] + cz * p[2][2]);
        }
    }
    // One record per (cell, object): the cell of the box centre, and every
    // cell the box touches (upper bound minus 1e-5); seq numbers the records
    // in object order.
    struct CellRec {
        int32_t x, y, z;
        uint32_t center;  // 1: the object's centre cell
        uint64_t seq;
        uint32_t touch;   // 1: the object's box touches the cell
        float size, ratio;
    };
    struct ObjCells {
        int lo[3], hi[3], cc[3];
        float avg, ratio;
    };
    std::vector<ObjCells> oc((size_t)nobj);
    std::vector<uint64_t> rstart((size_t)nobj + 1, 0);
#pragma omp parallel for schedule(static)
    for (int64_t o = 0; o < nobj; ++o) {
        const ObjStats& s = objs[o];
        if (!s.seen) continue;
        ObjCells& q = oc[o];
        float mesh_vol = std::fabs((float)s.volume) / 6.0f;
        float w = s.mx[0] - s.mn[0], h = s.mx[1] - s.mn[1], dpt = s.mx[2] - s.mn[2];
        float aabb_vol = w * h * dpt;
        if (aabb_vol < 1e-9f) aabb_vol = 1e-9f;
        float ratio = mesh_vol / aabb_vol;
        if (ratio > 1.0f) ratio = 1.0f;
        q.ratio = ratio;
        q.avg = (w + h + dpt) / 3.0f;
        uint64_t n = 1;
        for (int d = 0; d < 3; ++d) {
            const float c = (s.mn[d] + s.mx[d]) * 0.5f;
            q.cc[d] = (int)std::floor(c / cell_size);
            q.lo[d] = (int)std::floor(s.mn[d] / cell_size);
            q.hi[d] = (int)std::floor((s.mx[d] - 1e-5f) / cell_size);
            n *= (uint64_t)std::max<int64_t>(0, (int64_t)q.hi[d] - q.lo[d] + 1);
        }
        rstart[o + 1] = 1 + n;
    }
    for (int64_t o = 0; o < nobj; ++o) rstart[o + 1] += rstart[o];
    const uint64_t nrec = rstart[(size_t)nobj];
    std::unique_ptr<CellRec[]> recs(new CellRec[nrec]);
#pragma omp parallel for schedule(static)
    for (int64_t o = 0; o < nobj; ++o) {
        if (!objs[o].seen) continue;
        const ObjCells& q = oc[o];
        uint64_t r = rstart[o];
        recs[r] = CellRec{q.cc[0], q.cc[1], q.cc[2], 1u, r, 0u, 0.0f, 0.0f};
        ++r;
        for (int z = q.lo[2]; z <= q.hi[2]; ++z)
            for (int y = q.lo[1]; y <= q.hi[1]; ++y)
                for (int x = q.lo[0]; x <= q.hi[0]; ++x, ++r) recs[r] = CellRec{x, y, z, 0u, r, 1u, q.avg, q.ratio};
    }
    auto rec_less = [](const CellRec& a, const CellRec& b) {
        if (a.x != b.x) return a.x < b.x;
        if (a.y != b.y) return a.y < b.y;
        if (a.z != b.z) return a.z < b.z;
        return a.seq < b.seq;
    };
#ifdef _OPENMP
    __gnu_parallel::sort(recs.get(), recs.get() + nrec, rec_less);
#else
    std::sort(recs.get(), recs.get() + nrec, rec_less);
#endif
    g.grid_cells.clear();
    for (uint64_t i = 0; i < nrec;) {
        pierce_grid_entry e;
        e.ix = recs[i].x;
        e.iy = recs[i].y;
        e.iz = recs[i].z;
        uint32_t center = 0, touch = 0;
        float size = 0.0f, ratio = 0.0f;
        uint64_t j = i;
        for (; j < nrec && recs[j].x == e.ix && recs[j].y == e.iy && recs[j].z == e.iz; ++j) {
            center += recs[j].center;
            if (recs[j].touch) {
                touch++;
                size += recs[j].size;
                ratio += recs[j].ratio;
            }
        }
        e.center_count = center;
        e.touch_count = touch;
        e.avg_size_mean = size;
        e.vol_ratio = ratio;
        if (touch > 0) {
            e.avg_size_mean /= (float)touch;
            e.vol_ratio /= (float)touch;
        }
        g.grid_cells.push_back(e);
        i = j;
    }
    g.has_grid = true;
    g.grid_cell_size = cell_size;
}

}  // namespace pierce
