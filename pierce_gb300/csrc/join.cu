// Join kernels: edge-ray traversal, +Z parity rays, pair hash set,
// compaction, and the host orchestration of the overlap, intersection and
// containment joins.
//
// Edge rays (pierce/query/src/cuda/mesh_overlap_edges.cu:105-208): every
// unique edge of the source dataset is a closed segment; one thread per edge
// walks the target BVH with an exact box-overlap test (segment box vs child
// box, comparisons only) and tests the triangles of every reached leaf.  All
// hits are collected in a single traversal (the reference re-traces up to
// overlap_max_iterations times, advancing tmin past each hit).  Consecutive
// hits on one target object are emitted once.  Output modes: COUNT (hits per
// edge, pass 1 of the two-pass method), WRITE (keys at scanned offsets,
// pass 2), HASH (insert into the pair set, the reference's hash mode).
//
// Parity rays (mesh_intersection_anyhit.cu:46-240, mesh_containment.cu:
// 224-293): one thread per source object casts +Z from its first vertex and
// toggles the parity of (source, target-object) in a per-join parity table;
// odd entries are the "inside" pairs.
//
// Hash set (mesh_overlap_edges.cu:61-103): 64-bit keys (a << 32 | b), empty
// slot all ones, MurmurHash3 fmix64 finaliser, linear probing in a
// power-of-two table.  A probe sequence that exhausts its bound sets
// ERR_HASH_FULL instead of silently dropping the pair; the host then
// enlarges the table and reruns.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "predicates.cuh"

namespace pgpu {

enum RayMode { MODE_COUNT = 0, MODE_WRITE = 1, MODE_HASH = 2 };
enum Precision { PREC_EXACT = 0, PREC_FP32 = 1, PREC_DEFER = 2 };

constexpr int kShortStack = 32;  // stack entries kept in shared memory per thread (at most)
// default for culled edge rays against a per-join hierarchy: 8 entries
// (4 KB per block) leave more of the SM's shared memory / L1 to cache the
// hierarchy; deeper entries spill to local memory (2 % faster than 32 on the
// 2 x 50k ellipsoid join).  Unculled rays through a whole dataset's deeper
// hierarchy keep 32.
constexpr int kCulledShortStack = 8;

__device__ __forceinline__ uint64_t fmix64(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

__device__ __forceinline__ uint64_t pack_key(int32_t a, int32_t b) {
    return ((uint64_t)(uint32_t)a << 32) | (uint64_t)(uint32_t)b;
}

// Insert; returns slot index or -1 when the probe bound is exhausted.
// `probes` accumulates the slots inspected (for contention statistics).
__device__ __forceinline__ int64_t hash_insert(uint64_t* table, uint64_t mask, uint64_t key, uint32_t* err,
                                               uint32_t& probes) {
    uint64_t h = fmix64(key) & mask;
    for (uint64_t i = 0; i <= mask; ++i) {
        ++probes;
        const uint64_t cur = __ldcg(table + h);
        if (cur == key) return (int64_t)h;
        if (cur == kEmptyKey) {
            const unsigned long long old =
                atomicCAS(reinterpret_cast<unsigned long long*>(table + h), (unsigned long long)kEmptyKey,
                          (unsigned long long)key);
            if (old == kEmptyKey || old == key) return (int64_t)h;
        }
        h = (h + 1) & mask;
    }
    atomicOr(err, ERR_HASH_FULL);
    return -1;
}

__device__ __forceinline__ bool hash_contains(const uint64_t* table, uint64_t mask, uint64_t key) {
    uint64_t h = fmix64(key) & mask;
    for (uint64_t i = 0; i <= mask; ++i) {
        const uint64_t cur = __ldcg(table + h);
        if (cur == key) return true;
        if (cur == kEmptyKey) return false;
        h = (h + 1) & mask;
    }
    return false;
}

__device__ __forceinline__ bool sorted_contains(const uint64_t* keys, int64_t n, uint64_t key) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        const uint64_t v = keys[mid];
        if (v < key) lo = mid + 1;
        else hi = mid;
    }
    return lo < n && keys[lo] == key;
}

// Warp-aggregated counter flush: one atomicAdd per warp.
__device__ __forceinline__ void flush_counter(unsigned long long* dst, unsigned long long v) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, off);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}

struct EdgeRayParams {
    DevDataset src, tgt;
    int swap;
    int32_t* counts;
    const int64_t* offsets;
    uint64_t* keys;
    uint64_t* table;
    uint64_t mask;
    uint32_t* err;
    DevCounters* ctr;
    // optional compacted list of edges to trace (object culling)
    const uint32_t* ray_list;
    const unsigned long long* ray_count;
    unsigned long long* ray_cursor;
    // deferred exact tests: (edge << 32 | soup triangle) entries
    unsigned long long* amb_queue;
    unsigned long long* amb_count;
    uint64_t amb_cap;
    // tuning: rays a warp takes per fetch from the ray list, and traversal
    // stack entries kept in (dynamic) shared memory per thread
    int rays_per_fetch;
    int short_stack;
    int packets;  // 1: a warp traverses its 32 rays together (ray-list mode)
    // rays from triangles: list entries (t << 2 | k) name edge k of triangle
    // t of this soup (the source side's per-join hierarchy) instead of a
    // packed dataset edge
    const float4* ray_soup;
    int64_t ray_bound;  // ray indices of a listed launch lie below this
    // entry nodes of rays from a soup: ray_entry[t / entry_group] is the
    // four-wide target node every walk of soup triangle t's edges starts at
    // (group_entry); null: the root
    const int32_t* ray_entry;
    int entry_group;
    // shard k of n: dataset-edge rays with edge index in [E k / n,
    // E (k + 1) / n) of the source's E edges (ray lists from triangles hold
    // only the shard's rays already: k_soup_rays)
    int shard_index, shard_count;
};

// The segment of ray e and its source object: packed dataset edge e, or --
// with a ray soup -- edge k = e & 3 of soup triangle t = e >> 2: (v0, v1),
// (v1, v2) or (v2, v0), v0 carrying the object id.
// SOUP: 1 rays from a soup, 0 dataset edges, -1 decided by P.ray_soup at run time.
template <int SOUP = -1>
__device__ __forceinline__ void load_ray(const EdgeRayParams& P, int64_t e, float3& p, float3& q, int32_t& obj) {
    if (SOUP == 1 || (SOUP < 0 && P.ray_soup)) {
        const float4* tri = P.ray_soup + 3 * (e >> 2);
        const int k = (int)(e & 3);
        const float4 v0 = __ldg(tri);
        const float4 x = __ldg(tri + (k == 2 ? 2 : 1));  // v1 (k = 0, 1) or v2 (k = 2)
        obj = __float_as_int(v0.w);
        if (k == 0) {
            p = make_float3(v0.x, v0.y, v0.z);
            q = make_float3(x.x, x.y, x.z);
        } else if (k == 1) {
            const float4 v2 = __ldg(tri + 2);
            p = make_float3(x.x, x.y, x.z);
            q = make_float3(v2.x, v2.y, v2.z);
        } else {
            p = make_float3(x.x, x.y, x.z);
            q = make_float3(v0.x, v0.y, v0.z);
        }
        return;
    }
    const float4 s4 = __ldg(P.src.edges + 2 * e);
    const float4 e4 = __ldg(P.src.edges + 2 * e + 1);
    obj = __float_as_int(s4.w);
    p = make_float3(s4.x, s4.y, s4.z);
    q = make_float3(e4.x, e4.y, e4.z);
}

__device__ __forceinline__ bool box_overlap(float lx, float hx, float ly, float hy, float lz, float hz,
                                            const float3& lo, const float3& hi) {
    return lx <= hi.x && lo.x <= hx && ly <= hi.y && lo.y <= hy && lz <= hi.z && lo.z <= hz;
}

// Any-hit box query over a Node4 hierarchy from internal node `node`: true
// as soon as leaf_hit(first, count) is true for a leaf whose box meets
// [lo, hi] (and, conservatively, if the stack would overflow).
template <class LeafHit>
__device__ __forceinline__ bool any_hit4(const Node4* nodes4, int node, const float3& lo, const float3& hi,
                                         LeafHit&& leaf_hit) {
    int stack[kStackSize4];
    int sp = 0;
    for (;;) {
        const Node4* nd = nodes4 + node;
        const float4 lx = __ldg(&nd->lox), hx = __ldg(&nd->hix), ly = __ldg(&nd->loy), hy = __ldg(&nd->hiy);
        const float4 lz = __ldg(&nd->loz), hz = __ldg(&nd->hiz);
        const int4 ch = __ldg(&nd->ch);
        const int cnt = __ldg(&nd->meta.x);
        const bool h[4] = {box_overlap(lx.x, hx.x, ly.x, hy.x, lz.x, hz.x, lo, hi),
                           box_overlap(lx.y, hx.y, ly.y, hy.y, lz.y, hz.y, lo, hi),
                           box_overlap(lx.z, hx.z, ly.z, hy.z, lz.z, hz.z, lo, hi),
                           box_overlap(lx.w, hx.w, ly.w, hy.w, lz.w, hz.w, lo, hi)};
        const int c[4] = {ch.x, ch.y, ch.z, ch.w};
        int next = -1;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (!h[j]) continue;
            if (c[j] < 0) {
                if (leaf_hit(~c[j], (cnt >> (8 * j)) & 0xFF)) return true;
            } else if (next < 0) {
                next = c[j];
            } else {
                if (sp >= kStackSize4) return true;
                stack[sp++] = c[j];
            }
        }
        if (next >= 0) {
            node = next;
        } else {
            if (sp == 0) return false;
            node = stack[--sp];
        }
    }
}

struct RayCounters {
    uint32_t nodes = 0, tests = 0, hits = 0, inserts = 0, probes = 0;
};

// One edge ray against the target BVH.  PREC_EXACT resolves every test
// inline; PREC_DEFER classifies in float32 and queues undecided tests for
// k_resolve_ambiguous (the WRITE pass skips them: they were queued by the
// COUNT pass); PREC_FP32 is the plain Moller-Trumbore form.
// Where a traversal of tgt for source object src_obj starts: the root
// (node 0), a root leaf, or -- for partitioned datasets -- the subtree of the
// source object's partition.  Returns the start node, or -1 with the leaf
// range in (first, count) when the start is a leaf (count 0: nothing).
__device__ __forceinline__ int traversal_start(const DevDataset& src, const DevDataset& tgt, int32_t src_obj,
                                               int& first, int& count) {
    first = 0;
    count = 0;
    if (tgt.part_roots) {
        const int2 r = __ldg(tgt.part_roots + __ldg(src.obj_part + src_obj));
        if (r.x >= 0) return r.x;
        first = ~r.x;
        count = r.y;
        return -1;
    }
    if (tgt.root_is_leaf) {
        count = tgt.root_leaf_count;
        return -1;
    }
    return 0;
}

// The triangles [first, first + count) of a reached leaf against segment
// (p, q) with box [lo, hi]; hits of one target object in a row are emitted
// once (last_obj).
template <int MODE, int PREC>
__device__ __forceinline__ void leaf_tests(const EdgeRayParams& P, int64_t e, int first, int count, const float3& p,
                                           const float3& q, const float3& lo, const float3& hi, int32_t src_obj,
                                           int32_t& last_obj, int& nhit, int64_t& out, RayCounters& rc,
                                           PredCounters& pc) {
    for (int k = 0; k < count; ++k) {
        const int64_t t = (int64_t)first + k;
        const float4 a4 = __ldg(P.tgt.soup + 3 * t);
        const int32_t obj = __float_as_int(a4.w);
        if (obj == last_obj) continue;
        const float4 b4 = __ldg(P.tgt.soup + 3 * t + 1);
        const float4 c4 = __ldg(P.tgt.soup + 3 * t + 2);
        if (count > 1) {
            const float tlx = fminf(a4.x, fminf(b4.x, c4.x)), thx = fmaxf(a4.x, fmaxf(b4.x, c4.x));
            const float tly = fminf(a4.y, fminf(b4.y, c4.y)), thy = fmaxf(a4.y, fmaxf(b4.y, c4.y));
            const float tlz = fminf(a4.z, fminf(b4.z, c4.z)), thz = fmaxf(a4.z, fmaxf(b4.z, c4.z));
            if (!box_overlap(tlx, thx, tly, thy, tlz, thz, lo, hi)) continue;
        }
        ++rc.tests;
        const float3 a = make_float3(a4.x, a4.y, a4.z), b = make_float3(b4.x, b4.y, b4.z),
                     c = make_float3(c4.x, c4.y, c4.z);
        bool hit;
        if (PREC == PREC_EXACT) {
            hit = seg_tri_exact(p, q, a, b, c, pc);
        } else if (PREC == PREC_FP32) {
            hit = seg_tri_mt_fp32(p, q, a, b, c);
        } else {
            const int cls = seg_tri_fp32_class(p, q, a, b, c);
            if (cls == SEG_AMBIGUOUS) {
                ++pc.fp32_ambiguous;
                if (MODE != MODE_WRITE) {
                    const unsigned long long slot = atomicAdd(P.amb_count, 1ull);
                    if (slot < P.amb_cap) P.amb_queue[slot] = ((unsigned long long)e << 32) | (uint32_t)t;
                    else atomicOr(P.err, ERR_AMBIGUOUS_OVERFLOW);
                }
                continue;
            }
            hit = cls == SEG_HIT;
        }
        if (!hit) continue;
        last_obj = obj;
        ++nhit;
        if (MODE == MODE_COUNT) continue;
        const uint64_t key = P.swap ? pack_key(obj, src_obj) : pack_key(src_obj, obj);
        if (MODE == MODE_WRITE) {
            P.keys[out++] = key;
        } else {
            ++rc.inserts;
            hash_insert(P.table, P.mask, key, P.err, rc.probes);
        }
    }
}

// Ray e; `slot` indexes the per-ray counts and offsets of the two-pass
// method (the ray's position in the launch's ray list, or e without one).
template <int MODE, int PREC, bool WIDE = true, int SOUP = -1>
__device__ __forceinline__ void trace_edge(const EdgeRayParams& P, int64_t e, int64_t slot, int* sstack, int* lstack,
                                           RayCounters& rc, PredCounters& pc, int depth) {
    const int tid = threadIdx.x;
    float3 p, q;
    int32_t src_obj;
    load_ray<SOUP>(P, e, p, q, src_obj);
    const float3 lo = make_float3(fminf(p.x, q.x), fminf(p.y, q.y), fminf(p.z, q.z));
    const float3 hi = make_float3(fmaxf(p.x, q.x), fmaxf(p.y, q.y), fmaxf(p.z, q.z));
    int64_t out = (MODE == MODE_WRITE) ? P.offsets[slot] : 0;
    int32_t last_obj = -1;
    int nhit = 0;
    auto leaf = [&](int first, int count) {
        leaf_tests<MODE, PREC>(P, e, first, count, p, q, lo, hi, src_obj, last_obj, nhit, out, rc, pc);
    };
    int leaf_first, leaf_count;
    int node = traversal_start(P.src, P.tgt, src_obj, leaf_first, leaf_count);
    if (node < 0) {
        if (leaf_count > 0) leaf(leaf_first, leaf_count);
    } else if (WIDE && P.tgt.nodes4) {
        if (SOUP == 1 && P.ray_entry) node = __ldg(P.ray_entry + (uint32_t)(e >> 2) / (uint32_t)P.entry_group);
        // four-wide walk: a Node4 visit tests the four grandchildren of a
        // binary node, enters the first internal hit and pushes the others.
        // Reached leaves are queued (8 per thread) and tested when the queue
        // is full or the walk is over, so the lanes of a warp walk together
        // and test their leaves together (35 % less time than testing each
        // leaf when it is reached).
        constexpr int kPend = 8;
        uint64_t pend[kPend];
        int np = 0;
        auto flush = [&]() {
            for (int k = 0; k < np; ++k) leaf((int)(pend[k] >> 8), (int)(pend[k] & 0xFF));
            np = 0;
        };
        int sp = 0;
        for (;;) {
            ++rc.nodes;
            const Node4* nd = P.tgt.nodes4 + node;
            const float4 lx = __ldg(&nd->lox), hx = __ldg(&nd->hix), ly = __ldg(&nd->loy), hy = __ldg(&nd->hiy);
            const float4 lz = __ldg(&nd->loz), hz = __ldg(&nd->hiz);
            const int4 ch = __ldg(&nd->ch);
            const int cnt = __ldg(&nd->meta.x);
            const bool h[4] = {box_overlap(lx.x, hx.x, ly.x, hy.x, lz.x, hz.x, lo, hi),
                               box_overlap(lx.y, hx.y, ly.y, hy.y, lz.y, hz.y, lo, hi),
                               box_overlap(lx.z, hx.z, ly.z, hy.z, lz.z, hz.z, lo, hi),
                               box_overlap(lx.w, hx.w, ly.w, hy.w, lz.w, hz.w, lo, hi)};
            const int c[4] = {ch.x, ch.y, ch.z, ch.w};
            int next = -1;
            bool overflow = false;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (!h[j]) continue;
                if (c[j] < 0) {
                    if (np == kPend) flush();
                    pend[np++] = ((uint64_t)(uint32_t)(~c[j]) << 8) | (uint64_t)((cnt >> (8 * j)) & 0xFF);
                } else if (next < 0) {
                    next = c[j];
                } else if (sp >= kStackSize4) {
                    overflow = true;
                } else {
                    if (sp < depth) sstack[sp * 128 + tid] = c[j];
                    else lstack[sp - depth] = c[j];
                    ++sp;
                }
            }
            if (overflow) {
                atomicOr(P.err, ERR_STACK_OVERFLOW);
                break;
            }
            if (next >= 0) {
                node = next;
            } else {
                if (sp == 0) break;
                --sp;
                node = sp < depth ? sstack[sp * 128 + tid] : lstack[sp - depth];
            }
        }
        flush();
    } else {
        int sp = 0;
        for (;;) {
            ++rc.nodes;
            const Node* nd = P.tgt.nodes + node;
            const float4 bx = __ldg(&nd->bx), by = __ldg(&nd->by), bz = __ldg(&nd->bz);
            const int4 ch = __ldg(&nd->ch);
            bool h0 = box_overlap(bx.x, bx.y, by.x, by.y, bz.x, bz.y, lo, hi);
            bool h1 = box_overlap(bx.z, bx.w, by.z, by.w, bz.z, bz.w, lo, hi);
            if (h0 && ch.x < 0) {
                leaf(~ch.x, ch.z & 0xFF);
                h0 = false;
            }
            if (h1 && ch.y < 0) {
                leaf(~ch.y, (ch.z >> 8) & 0xFF);
                h1 = false;
            }
            if (h0 && h1) {
                if (sp >= kStackSize) {
                    atomicOr(P.err, ERR_STACK_OVERFLOW);
                    break;
                }
                if (sp < depth) sstack[sp * 128 + tid] = ch.y;
                else lstack[sp - depth] = ch.y;
                ++sp;
                node = ch.x;
            } else if (h0) {
                node = ch.x;
            } else if (h1) {
                node = ch.y;
            } else {
                if (sp == 0) break;
                --sp;
                node = sp < depth ? sstack[sp * 128 + tid] : lstack[sp - depth];
            }
        }
    }
    if (MODE == MODE_COUNT) P.counts[slot] = nhit;
    rc.hits += (uint32_t)nhit;
}

// Warp-cooperative traversal of 32 rays (one per lane, e < 0: none).  The
// rays of a fetch come from one 32-edge chunk, so they are close together:
// the warp walks the hierarchy once, each node is loaded once for all lanes
// (one broadcast load), every lane tests its own segment against the two
// child boxes, and a child is entered with the mask of the lanes that meet
// it (__ballot_sync).  The node stack (node, lane mask) is shared by the
// warp.  Leaves are tested per lane with the same code as trace_edge, so the
// hits of each ray equal those of the one-ray-per-thread traversal.  When
// the lanes start in different subtrees (partitions) each lane falls back
// to the one-ray traversal with a local stack.
template <int MODE, int PREC, int SOUP = -1>
__device__ __forceinline__ void trace_packet(const EdgeRayParams& P, int64_t e, int64_t slot, int2* wstack,
                                             int* lstack, RayCounters& rc, PredCounters& pc) {
    const int lane = threadIdx.x & 31;
    const bool valid = e >= 0;
    const unsigned vmask = __ballot_sync(0xFFFFFFFFu, valid);
    if (!vmask) return;
    float3 p = make_float3(0, 0, 0), q = make_float3(0, 0, 0);
    int32_t src_obj = 0;
    if (valid) load_ray<SOUP>(P, e, p, q, src_obj);
    int lf = 0, lc = 0;
    const int node0 = valid ? traversal_start(P.src, P.tgt, src_obj, lf, lc) : 0;
    const int leader = __ffs(vmask) - 1;
    const int n0 = __shfl_sync(0xFFFFFFFFu, node0, leader);
    const int lf0 = __shfl_sync(0xFFFFFFFFu, lf, leader), lc0 = __shfl_sync(0xFFFFFFFFu, lc, leader);
    const bool same = __all_sync(0xFFFFFFFFu, !valid || (node0 == n0 && (n0 >= 0 || (lf == lf0 && lc == lc0))));
    if (!same) {
        if (valid) trace_edge<MODE, PREC, true, SOUP>(P, e, slot, nullptr, lstack, rc, pc, 0);
        return;
    }
    const float3 lo = make_float3(fminf(p.x, q.x), fminf(p.y, q.y), fminf(p.z, q.z));
    const float3 hi = make_float3(fmaxf(p.x, q.x), fmaxf(p.y, q.y), fmaxf(p.z, q.z));
    int64_t out = (MODE == MODE_WRITE && valid) ? P.offsets[slot] : 0;
    int32_t last_obj = -1;
    int nhit = 0;
    auto leaf = [&](int first, int count) {
        leaf_tests<MODE, PREC>(P, e, first, count, p, q, lo, hi, src_obj, last_obj, nhit, out, rc, pc);
    };
    if (n0 < 0) {
        if (valid && lc0 > 0) leaf(lf0, lc0);
    } else {
        int node = n0, sp = 0;
        unsigned mask = vmask;
        for (;;) {
            if (lane == 0) ++rc.nodes;
            const Node* nd = P.tgt.nodes + node;
            const float4 bx = __ldg(&nd->bx), by = __ldg(&nd->by), bz = __ldg(&nd->bz);
            const int4 ch = __ldg(&nd->ch);
            const bool in = (mask >> lane) & 1u;
            const bool h0 = in && box_overlap(bx.x, bx.y, by.x, by.y, bz.x, bz.y, lo, hi);
            const bool h1 = in && box_overlap(bx.z, bx.w, by.z, by.w, bz.z, bz.w, lo, hi);
            unsigned m0 = __ballot_sync(0xFFFFFFFFu, h0), m1 = __ballot_sync(0xFFFFFFFFu, h1);
            if (ch.x < 0 && m0) {
                if (h0) leaf(~ch.x, ch.z & 0xFF);
                m0 = 0;
            }
            if (ch.y < 0 && m1) {
                if (h1) leaf(~ch.y, (ch.z >> 8) & 0xFF);
                m1 = 0;
            }
            __syncwarp();
            if (m0 && m1) {
                if (sp >= kStackSize) {
                    if (lane == 0) atomicOr(P.err, ERR_STACK_OVERFLOW);
                    break;
                }
                if (lane == 0) wstack[sp] = make_int2(ch.y, (int)m1);
                ++sp;
                node = ch.x;
                mask = m0;
            } else if (m0) {
                node = ch.x;
                mask = m0;
            } else if (m1) {
                node = ch.y;
                mask = m1;
            } else {
                if (sp == 0) break;
                --sp;
                __syncwarp();
                const int2 top = wstack[sp];
                node = top.x;
                mask = (unsigned)top.y;
            }
            __syncwarp();
        }
    }
    if (valid) {
        if (MODE == MODE_COUNT) P.counts[slot] = nhit;
        rc.hits += (uint32_t)nhit;
    }
}

// FORM 1: the culled ray list, one ray per thread (four-wide or binary
// walk); FORM 2: the culled ray list in warp packets; FORM 0: one thread per
// edge over a binary hierarchy (the unculled plain form).  Each form is its
// own kernel, so none carries the registers of another's code.
// SOUP (listed forms): 1 rays from the source side's per-join soup, 0 the
// dataset's edges, each its own instantiation (no registers for the other).
// The one-ray-per-thread walk over a list (FORM 1) with the FP32 filter
// keeps 8 blocks of 128 per SM resident (64 registers).
template <int MODE, int PREC, int FORM, int SOUP>
__global__ void __launch_bounds__(128, (FORM == 1 && PREC != PREC_EXACT) ? 8 : 1) k_edge_rays(EdgeRayParams P) {
    extern __shared__ int sstack[];  // short_stack x 128 entries (then per-form data)
    int lstack[FORM ? kStackSize4 : kStackSize];
    RayCounters rc;
    PredCounters pc{0, 0};
    uint32_t rays = 0;
    if (FORM) {
        // Compacted ray list, persistent blocks: each warp takes the next
        // rays_per_fetch rays from a global cursor (the work queue), so uneven
        // ray costs balance out.
        const unsigned long long n = *P.ray_count;
        // the shard of a dataset-edge ray depends on its edge index only, not
        // on its position in the list (whose order varies between runs)
        const bool by_edge = P.shard_count > 1 && !P.ray_soup;
        const int64_t elo = P.src.num_edges * P.shard_index / P.shard_count;
        const int64_t ehi = P.src.num_edges * (P.shard_index + 1) / P.shard_count;
        const int lane = threadIdx.x & 31;
        const unsigned long long per = (unsigned long long)P.rays_per_fetch;
        int2* wstack = reinterpret_cast<int2*>(sstack + P.short_stack * 128) + (threadIdx.x >> 5) * kStackSize;
        for (;;) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(P.ray_cursor, per);
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base >= n) break;
            for (unsigned long long r = lane; r < per; r += 32) {  // per/32 rounds for every lane
                const unsigned long long i = base + r;
                const int64_t e = i < n ? (int64_t)P.ray_list[i] : -1;
                const bool mine = e >= 0 && (!by_edge || (e >= elo && e < ehi));
                if (FORM == 2) {
                    trace_packet<MODE, PREC, SOUP>(P, mine ? e : -1, (int64_t)i, wstack, lstack, rc, pc);
                    rays += mine ? 1u : 0u;
                } else if (mine) {
                    trace_edge<MODE, PREC, true, SOUP>(P, e, (int64_t)i, sstack, lstack, rc, pc, P.short_stack);
                    ++rays;
                }
            }
        }
    } else {
        const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
        const int64_t lo = P.src.num_edges * P.shard_index / P.shard_count;
        const int64_t hi = P.src.num_edges * (P.shard_index + 1) / P.shard_count;
        if (e >= lo && e < hi) {
            trace_edge<MODE, PREC, false, 0>(P, e, e, sstack, lstack, rc, pc, P.short_stack);
            ++rays;
        }
    }
    flush_counter(&P.ctr->rays, rays);
    flush_counter(&P.ctr->node_visits, rc.nodes);
    flush_counter(&P.ctr->tri_tests, rc.tests);
    flush_counter(&P.ctr->raw_hits, rc.hits);
    flush_counter(&P.ctr->fp32_ambiguous, pc.fp32_ambiguous);
    flush_counter(&P.ctr->fp64_ambiguous, pc.fp64_ambiguous);
    if (MODE == MODE_HASH) {
        flush_counter(&P.ctr->hash_accesses, rc.probes);
        flush_counter(&P.ctr->hash_contentions, rc.probes - rc.inserts);
    }
}

// Exact resolution of the queued (edge, triangle) tests.  Hits go to the
// hash set (table != null) or are appended to keys_out.
__global__ void __launch_bounds__(128) k_resolve_ambiguous(EdgeRayParams P, uint64_t* keys_out,
                                                           unsigned long long* keys_count, uint64_t keys_cap) {
    PredCounters pc{0, 0};
    uint32_t probes = 0, inserts = 0;
    const unsigned long long n = min(*P.amb_count, (unsigned long long)P.amb_cap);
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long ent = P.amb_queue[i];
        const int64_t e = (int64_t)(ent >> 32), t = (int64_t)(ent & 0xFFFFFFFFull);
        float3 p, q;
        int32_t src_obj;
        load_ray(P, e, p, q, src_obj);
        const float4 a4 = __ldg(P.tgt.soup + 3 * t), b4 = __ldg(P.tgt.soup + 3 * t + 1),
                     c4 = __ldg(P.tgt.soup + 3 * t + 2);
        if (!seg_tri_exact(p, q, make_float3(a4.x, a4.y, a4.z), make_float3(b4.x, b4.y, b4.z),
                           make_float3(c4.x, c4.y, c4.z), pc))
            continue;
        const int32_t obj = __float_as_int(a4.w);
        const uint64_t key = P.swap ? pack_key(obj, src_obj) : pack_key(src_obj, obj);
        if (P.table) {
            ++inserts;
            hash_insert(P.table, P.mask, key, P.err, probes);
        } else {
            const unsigned long long pos = atomicAdd(keys_count, 1ull);
            if (pos < keys_cap) keys_out[pos] = key;
            else atomicOr(P.err, ERR_OUTPUT_OVERFLOW);
        }
    }
    // fp32_ambiguous is counted by the tracing kernel; here only escalations to exact
    flush_counter(&P.ctr->fp64_ambiguous, pc.fp64_ambiguous);
    flush_counter(&P.ctr->hash_accesses, probes);
    flush_counter(&P.ctr->hash_contentions, probes - inserts);
}

// Object culling: a source object is active when its box overlaps the box
// of at least one target triangle (exact comparisons).  A segment's box lies
// inside its object's box, so inactive objects' edges cannot hit anything.
__global__ void __launch_bounds__(128) k_object_active(DevDataset src, DevDataset tgt, uint8_t* active) {
    __shared__ int sstack[kShortStack][128];
    int lstack[kStackSize - kShortStack];
    const int tid = threadIdx.x;
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + tid;
    if (o >= src.num_objects) return;
    const float* b = src.obj_box + 6 * o;
    const float3 lo = make_float3(b[0], b[1], b[2]), hi = make_float3(b[3], b[4], b[5]);
    bool found = false;
    if (lo.x <= hi.x && tgt.num_tris > 0) {
        auto leaf = [&](int first, int count) {
            for (int k = 0; k < count && !found; ++k) {
                const int64_t t = (int64_t)first + k;
                const float4 a4 = __ldg(tgt.soup + 3 * t), b4 = __ldg(tgt.soup + 3 * t + 1),
                             c4 = __ldg(tgt.soup + 3 * t + 2);
                found = box_overlap(fminf(a4.x, fminf(b4.x, c4.x)), fmaxf(a4.x, fmaxf(b4.x, c4.x)),
                                    fminf(a4.y, fminf(b4.y, c4.y)), fmaxf(a4.y, fmaxf(b4.y, c4.y)),
                                    fminf(a4.z, fminf(b4.z, c4.z)), fmaxf(a4.z, fmaxf(b4.z, c4.z)), lo, hi);
            }
        };
        int leaf_first, leaf_count;
        int node = traversal_start(src, tgt, (int32_t)o, leaf_first, leaf_count);
        if (node < 0) {
            leaf(leaf_first, leaf_count);
        } else if (tgt.nodes4) {
            found = any_hit4(tgt.nodes4, node, lo, hi, [&](int first, int count) {
                leaf(first, count);
                return found;
            });
        } else {
            int sp = 0;
            while (!found) {
                const Node* nd = tgt.nodes + node;
                const float4 bx = __ldg(&nd->bx), by = __ldg(&nd->by), bz = __ldg(&nd->bz);
                const int4 ch = __ldg(&nd->ch);
                bool h0 = box_overlap(bx.x, bx.y, by.x, by.y, bz.x, bz.y, lo, hi);
                bool h1 = box_overlap(bx.z, bx.w, by.z, by.w, bz.z, bz.w, lo, hi);
                if (h0 && ch.x < 0) {
                    leaf(~ch.x, ch.z & 0xFF);
                    h0 = false;
                }
                if (!found && h1 && ch.y < 0) {
                    leaf(~ch.y, (ch.z >> 8) & 0xFF);
                    h1 = false;
                }
                if (found) break;
                if (h0 && h1) {
                    if (sp >= kStackSize) {  // cannot happen for an LBVH; be conservative
                        found = true;
                        break;
                    }
                    if (sp < kShortStack) sstack[sp][tid] = ch.y;
                    else lstack[sp - kShortStack] = ch.y;
                    ++sp;
                    node = ch.x;
                } else if (h0) {
                    node = ch.x;
                } else if (h1) {
                    node = ch.y;
                } else {
                    if (sp == 0) break;
                    --sp;
                    node = sp < kShortStack ? sstack[sp][tid] : lstack[sp - kShortStack];
                }
            }
        }
    }
    active[o] = found ? 1 : 0;
}

// Block-aggregated stream compaction: each thread takes ITEMS consecutive
// elements of a tile, the block scans its keep counts in shared memory and
// reserves its output range with one atomicAdd per tile, so a single
// counter sees one atomic per blockDim*ITEMS elements.
template <int ITEMS, class Keep>
__device__ __forceinline__ void compact_tiles(int64_t n, Keep keep, uint32_t* __restrict__ out,
                                              unsigned long long* count) {
    __shared__ uint32_t warp_tot[32];
    __shared__ unsigned long long block_base;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nwarps = blockDim.x >> 5;
    const int64_t tile = (int64_t)blockDim.x * ITEMS;
    for (int64_t base = (int64_t)blockIdx.x * tile; base < n; base += (int64_t)gridDim.x * tile) {
        const int64_t first = base + (int64_t)tid * ITEMS;
        uint32_t mask = 0;
#pragma unroll
        for (int k = 0; k < ITEMS; ++k)
            if (first + k < n && keep(first + k)) mask |= 1u << k;
        const uint32_t c = __popc(mask);
        uint32_t incl = c;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, off);
            if (lane >= off) incl += v;
        }
        if (lane == 31) warp_tot[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            uint32_t w = lane < nwarps ? warp_tot[lane] : 0;
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, w, off);
                if (lane >= off) w += v;
            }
            if (lane < nwarps) warp_tot[lane] = w;  // inclusive over warps
            if (lane == 31) block_base = w ? atomicAdd(count, (unsigned long long)w) : 0ull;
        }
        __syncthreads();
        unsigned long long pos = block_base + (wid ? warp_tot[wid - 1] : 0u) + (incl - c);
#pragma unroll
        for (int k = 0; k < ITEMS; ++k)
            if (mask & (1u << k)) out[pos++] = (uint32_t)(first + k);
        __syncthreads();
    }
}

// Edges of active objects -> compacted list.
__global__ void __launch_bounds__(256) k_collect_rays(const int32_t* __restrict__ edge_src, int64_t n,
                                                      const uint8_t* __restrict__ active, uint32_t* __restrict__ list,
                                                      unsigned long long* count) {
    compact_tiles<8>(n, [&](int64_t e) { return active[edge_src[e]] != 0; }, list, count);
}

struct ParityParams {
    DevDataset src, tgt;
    int64_t src_lo, src_hi;  // source objects [src_lo, src_hi) cast rays (a shard)
    int swap;
    uint64_t* table;
    uint32_t* parity;
    uint64_t mask;
    uint32_t* err;
    DevCounters* ctr;
};

__global__ void __launch_bounds__(128) k_parity(ParityParams P) {
    __shared__ int sstack[kShortStack][128];
    int lstack[kStackSize - kShortStack];
    const int tid = threadIdx.x;
    uint32_t n_nodes = 0, n_tests = 0, n_cross = 0;
    PredCounters pc{0, 0};
    const int64_t o = P.src_lo + blockIdx.x * (int64_t)blockDim.x + tid;
    bool active = o < P.src_hi;
    if (active) {
        const float4 fv = __ldg(P.src.first_vertex + o);
        active = fv.w == 0.0f;
        const float3 p = make_float3(fv.x, fv.y, fv.z);
        auto leaf = [&](int first, int count) {
            for (int k = 0; k < count; ++k) {
                const int64_t t = (int64_t)first + k;
                const float4 a4 = __ldg(P.tgt.soup + 3 * t), b4 = __ldg(P.tgt.soup + 3 * t + 1),
                             c4 = __ldg(P.tgt.soup + 3 * t + 2);
                if (count > 1) {
                    if (fminf(a4.x, fminf(b4.x, c4.x)) > p.x || fmaxf(a4.x, fmaxf(b4.x, c4.x)) < p.x ||
                        fminf(a4.y, fminf(b4.y, c4.y)) > p.y || fmaxf(a4.y, fmaxf(b4.y, c4.y)) < p.y ||
                        fmaxf(a4.z, fmaxf(b4.z, c4.z)) < p.z)
                        continue;
                }
                ++n_tests;
                if (!zray_cross(p, make_float3(a4.x, a4.y, a4.z), make_float3(b4.x, b4.y, b4.z),
                                make_float3(c4.x, c4.y, c4.z), pc))
                    continue;
                ++n_cross;
                const int32_t obj = __float_as_int(a4.w);
                const uint64_t key = P.swap ? pack_key(obj, (int32_t)o) : pack_key((int32_t)o, obj);
                uint32_t probes = 0;
                const int64_t slot = hash_insert(P.table, P.mask, key, P.err, probes);
                if (slot >= 0) P.parity[slot] ^= 1u;  // keys of one source are owned by one thread
            }
        };
        if (active) {
            int leaf_first, leaf_count;
            int node = traversal_start(P.src, P.tgt, (int32_t)o, leaf_first, leaf_count);
            if (node < 0) {
                if (leaf_count > 0) leaf(leaf_first, leaf_count);
            } else {
                int sp = 0;
                for (;;) {
                    ++n_nodes;
                    const Node* nd = P.tgt.nodes + node;
                    const float4 bx = __ldg(&nd->bx), by = __ldg(&nd->by), bz = __ldg(&nd->bz);
                    const int4 ch = __ldg(&nd->ch);
                    bool h0 = bx.x <= p.x && p.x <= bx.y && by.x <= p.y && p.y <= by.y && bz.y >= p.z;
                    bool h1 = bx.z <= p.x && p.x <= bx.w && by.z <= p.y && p.y <= by.w && bz.w >= p.z;
                    if (h0 && ch.x < 0) {
                        leaf(~ch.x, ch.z & 0xFF);
                        h0 = false;
                    }
                    if (h1 && ch.y < 0) {
                        leaf(~ch.y, (ch.z >> 8) & 0xFF);
                        h1 = false;
                    }
                    if (h0 && h1) {
                        if (sp >= kStackSize) {
                            atomicOr(P.err, ERR_STACK_OVERFLOW);
                            break;
                        }
                        if (sp < kShortStack) sstack[sp][tid] = ch.y;
                        else lstack[sp - kShortStack] = ch.y;
                        ++sp;
                        node = ch.x;
                    } else if (h0) {
                        node = ch.x;
                    } else if (h1) {
                        node = ch.y;
                    } else {
                        if (sp == 0) break;
                        --sp;
                        node = sp < kShortStack ? sstack[sp][tid] : lstack[sp - kShortStack];
                    }
                }
            }
        }
    }
    flush_counter(&P.ctr->parity_rays, active ? 1ull : 0ull);
    flush_counter(&P.ctr->node_visits, n_nodes);
    flush_counter(&P.ctr->tri_tests, n_tests);
    flush_counter(&P.ctr->fp32_ambiguous, pc.fp32_ambiguous);
    flush_counter(&P.ctr->fp64_ambiguous, pc.fp64_ambiguous);
    (void)n_cross;
}

// Odd-parity entries of a parity table.  mode 0: insert into out_table;
// mode 1 (containment): keep only keys absent from the overlap set (hash
// table or sorted array) and append them to out_keys.
__global__ void k_parity_emit(const uint64_t* __restrict__ ptable, const uint32_t* __restrict__ parity, uint64_t pslots,
                              int mode, const uint64_t* lookup_table, uint64_t lookup_mask,
                              const uint64_t* lookup_sorted, int64_t lookup_n, uint64_t* out_table, uint64_t out_mask,
                              uint64_t* out_keys, unsigned long long* out_count, uint64_t out_cap, uint32_t* err) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < pslots; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t key = ptable[i];
        if (key == kEmptyKey || !(parity[i] & 1u)) continue;
        if (mode == 1) {
            const bool in = lookup_table ? hash_contains(lookup_table, lookup_mask, key)
                                         : sorted_contains(lookup_sorted, lookup_n, key);
            if (in) continue;
        }
        if (out_table) {
            uint32_t probes = 0;
            hash_insert(out_table, out_mask, key, err, probes);
        } else {
            const unsigned long long pos = atomicAdd(out_count, 1ull);
            if (pos < out_cap) out_keys[pos] = key;
        }
    }
}

// Containment candidates: the objects of the odd (a, b) entries of a parity
// table (key a << 32 | b).  Activity flags are 0 or 1; a candidate's flag
// gains bit 1 (only ever OR-ed in, so concurrent stores of one byte agree),
// then k_keep_candidates keeps the objects that are both active and
// candidates.
__global__ void k_mark_candidates(const uint64_t* __restrict__ ptable, const uint32_t* __restrict__ parity,
                                  uint64_t pslots, uint8_t* act_a, uint8_t* act_b) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < pslots; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t key = ptable[i];
        if (key == kEmptyKey || !(parity[i] & 1u)) continue;
        const uint32_t a = (uint32_t)(key >> 32), b = (uint32_t)key;
        act_a[a] = (uint8_t)(act_a[a] | 2u);
        act_b[b] = (uint8_t)(act_b[b] | 2u);
    }
}

__global__ void k_keep_candidates(uint8_t* flags, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        flags[i] = flags[i] == 3u ? 1u : 0u;
}

// ---- containment by candidate pairs -------------------------------------------
// Containment is parity(B in A) \ overlap (pierce_containment_main.cpp:
// 385-550), so only the odd-parity pairs (a, b) need an overlap answer.  A
// block of kPairThreads takes one such pair, so that one large pair does
// not hold a lone warp for the whole launch: it lists the triangles of a
// (those of a's 32-triangle chunks whose boxes meet, read first) whose boxes
// meet the intersection of the two object boxes (a patch of a's
// surface; the vertices of up to kPairVerts of them are kept in shared
// memory), shrinks the box to that patch's box, and streams b's triangles
// past them, one per thread (a triangle whose 32-triangle chunk box misses
// the patch is skipped unread), each tested against the listed triangles whose
// boxes meet its own with the exact closed triangle-triangle predicate (an
// edge of one meets the other: six segment tests, the edge definition for
// the edges of triangles).  The pair is a containment pair when none meets;
// a b deep inside a lists nothing and costs one pass over a's triangles.  A
// patch larger than kPairList is read from a's range in place.  A pair whose
// objects hold more than kPairScanMax triangles together, or whose unlisted
// patch would cost more than kPairStreamMax triangle pairs, is counted in
// *fallback and the join takes the culling pipeline instead.
constexpr int kPairThreads = 256;
constexpr int kPairList = 1024;
constexpr int kPairVerts = 512;
constexpr int kPairChunkList = 512;  // listed chunks of the container (more: its whole range)
constexpr int kPairScanMax = 1 << 16;
constexpr int64_t kPairStreamMax = 1 << 22;

struct PairParams {
    const uint64_t* ptable;
    const uint32_t* parity;
    uint64_t pslots;
    DevDataset a, b;  // vertices, indices, object ranges and boxes
    uint64_t* out;
    unsigned long long* count;
    uint64_t cap;
    unsigned long long* fallback;
    DevCounters* ctr;
};

__device__ __forceinline__ float3 tri_vertex(const DevDataset& d, uint32_t tri, int k) {
    const uint32_t i = __ldg(d.idx + 3 * (size_t)tri + k);
    return make_float3(__ldg(d.verts + 3 * (size_t)i), __ldg(d.verts + 3 * (size_t)i + 1),
                       __ldg(d.verts + 3 * (size_t)i + 2));
}

__device__ __forceinline__ bool tri_box_meets(const float3& p, const float3& q, const float3& r, const float3& lo,
                                              const float3& hi) {
    return box_overlap(fminf(p.x, fminf(q.x, r.x)), fmaxf(p.x, fmaxf(q.x, r.x)), fminf(p.y, fminf(q.y, r.y)),
                       fmaxf(p.y, fmaxf(q.y, r.y)), fminf(p.z, fminf(q.z, r.z)), fmaxf(p.z, fmaxf(q.z, r.z)), lo, hi);
}

__device__ __forceinline__ float block_min(float v, float* red) {
    for (int off = 16; off; off >>= 1) v = fminf(v, __shfl_xor_sync(0xFFFFFFFFu, v, off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float r = red[0];
    for (int k = 1; k < kPairThreads / 32; ++k) r = fminf(r, red[k]);
    __syncthreads();
    return r;
}
__device__ __forceinline__ float block_max(float v, float* red) { return -block_min(-v, red); }

// Position of this thread's flag among the block's set flags, after `base`
// (warp ballots; per-warp counts in s_warp), and the block's total.
__device__ __forceinline__ int block_compact(bool flag, int base, int* s_warp) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, flag);
    if (lane == 0) s_warp[w] = __popc(m);
    __syncthreads();
    int before = base;
    for (int q = 0; q < w; ++q) before += s_warp[q];
    return before + __popc(m & ((1u << lane) - 1u));
}
__device__ __forceinline__ int block_total(const int* s_warp) {
    int total = 0;
    for (int q = 0; q < kPairThreads / 32; ++q) total += s_warp[q];
    return total;
}

__global__ void __launch_bounds__(kPairThreads) k_containment_pairs(PairParams P) {
    __shared__ uint32_t s_list[kPairList];
    __shared__ uint32_t s_chunk[kPairChunkList];
    __shared__ float4 s_tri[kPairVerts][3];
    __shared__ int s_warp[kPairThreads / 32];
    __shared__ float s_red[kPairThreads / 32];
    __shared__ uint64_t s_pairs[kPairThreads];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    PredCounters pc{0, 0};
    uint32_t tests = 0;
    // windows of kPairThreads slots of the parity table: every thread reads
    // one slot, the block compacts the odd pairs, then takes them in turn
    for (int64_t wbase = (int64_t)blockIdx.x * kPairThreads; wbase < (int64_t)P.pslots;
         wbase += (int64_t)gridDim.x * kPairThreads) {
        uint64_t slot_key = kEmptyKey;
        bool odd = false;
        if (wbase + tid < (int64_t)P.pslots) {
            slot_key = P.ptable[wbase + tid];
            odd = slot_key != kEmptyKey && (P.parity[wbase + tid] & 1u);
        }
        const int odd_pos = block_compact(odd, 0, s_warp);
        const int n_odd = block_total(s_warp);
        if (odd) s_pairs[odd_pos] = slot_key;
        __syncthreads();
        for (int q = 0; q < n_odd; ++q) {
            const uint64_t key = s_pairs[q];
            const uint32_t a = (uint32_t)(key >> 32), b = (uint32_t)key;
            const float* ba = P.a.obj_box + 6 * (size_t)a;
            const float* bb = P.b.obj_box + 6 * (size_t)b;
            float3 lo = make_float3(fmaxf(__ldg(ba), __ldg(bb)), fmaxf(__ldg(ba + 1), __ldg(bb + 1)),
                                    fmaxf(__ldg(ba + 2), __ldg(bb + 2)));
            float3 hi = make_float3(fminf(__ldg(ba + 3), __ldg(bb + 3)), fminf(__ldg(ba + 4), __ldg(bb + 4)),
                                    fminf(__ldg(ba + 5), __ldg(bb + 5)));
            bool meets = false, undecided = false;
            if (lo.x <= hi.x && lo.y <= hi.y && lo.z <= hi.z) {
                const int2 ra = __ldg(P.a.obj_range + a), rb = __ldg(P.b.obj_range + b);
                if ((int64_t)ra.y + rb.y > kPairScanMax) {
                    undecided = true;
                } else {
                    // a's 32-triangle chunks whose boxes meet the common box, then
                    // the triangles of those chunks that do: the list (block-wide
                    // compaction) and the patch box
                    const int c0 = ra.x >> 5, c1 = (ra.x + ra.y - 1) >> 5;
                    int nmc = 0;
                    for (int base = c0; base <= c1; base += kPairThreads) {
                        const int c = base + tid;
                        bool meet = true;  // no chunk boxes: every chunk
                        if (c > c1) meet = false;
                        else if (P.a.tri_chunk_box) {
                            const float* cb = P.a.tri_chunk_box + 6 * (size_t)c;
                            meet = box_overlap(__ldg(cb), __ldg(cb + 3), __ldg(cb + 1), __ldg(cb + 4), __ldg(cb + 2),
                                               __ldg(cb + 5), lo, hi);
                        }
                        const int pos = block_compact(meet, nmc, s_warp);
                        if (meet && pos < kPairChunkList) s_chunk[pos] = (uint32_t)c;
                        nmc += block_total(s_warp);
                        __syncthreads();
                    }
                    int na = 0;
                    float3 plo = make_float3(3.4e38f, 3.4e38f, 3.4e38f), phi = make_float3(-3.4e38f, -3.4e38f, -3.4e38f);
                    const bool by_chunks = nmc <= kPairChunkList;
                    const int slots = by_chunks ? 32 * nmc : ra.y;
                    for (int base = 0; base < slots; base += kPairThreads) {
                        const int k = base + tid;
                        bool meet = false;
                        uint32_t t = 0;
                        if (k < slots) {
                            const int tt = by_chunks ? (int)(s_chunk[k >> 5] << 5) + (k & 31) : ra.x + k;
                            if (tt >= ra.x && tt < ra.x + ra.y) {
                                t = (uint32_t)tt;
                                const float3 v0 = tri_vertex(P.a, t, 0), v1 = tri_vertex(P.a, t, 1),
                                             v2 = tri_vertex(P.a, t, 2);
                                meet = tri_box_meets(v0, v1, v2, lo, hi);
                                if (meet) {
                                    plo = make_float3(fminf(plo.x, fminf(v0.x, fminf(v1.x, v2.x))),
                                                      fminf(plo.y, fminf(v0.y, fminf(v1.y, v2.y))),
                                                      fminf(plo.z, fminf(v0.z, fminf(v1.z, v2.z))));
                                    phi = make_float3(fmaxf(phi.x, fmaxf(v0.x, fmaxf(v1.x, v2.x))),
                                                      fmaxf(phi.y, fmaxf(v0.y, fmaxf(v1.y, v2.y))),
                                                      fmaxf(phi.z, fmaxf(v0.z, fmaxf(v1.z, v2.z))));
                                }
                            }
                        }
                        const int pos = block_compact(meet, na, s_warp);
                        if (meet && pos < kPairList) s_list[pos] = t;
                        na += block_total(s_warp);
                        __syncthreads();
                    }
                    plo = make_float3(block_min(plo.x, s_red), block_min(plo.y, s_red), block_min(plo.z, s_red));
                    phi = make_float3(block_max(phi.x, s_red), block_max(phi.y, s_red), block_max(phi.z, s_red));
                    const bool listed = na <= kPairList;
                    const bool cached = na <= kPairVerts;
                    if (cached) {
                        for (int k = tid; k < na; k += kPairThreads) {
                            const uint32_t t = s_list[k];
                            for (int v = 0; v < 3; ++v) {
                                const float3 x = tri_vertex(P.a, t, v);
                                s_tri[k][v] = make_float4(x.x, x.y, x.z, 0.0f);
                            }
                        }
                        __syncthreads();
                    }
                    if (!listed && (int64_t)ra.y * rb.y > kPairStreamMax) {
                        undecided = true;
                    } else if (na > 0) {
                        lo = make_float3(fmaxf(lo.x, plo.x), fmaxf(lo.y, plo.y), fmaxf(lo.z, plo.z));
                        hi = make_float3(fminf(hi.x, phi.x), fminf(hi.y, phi.y), fminf(hi.z, phi.z));
                        const int nj = listed ? na : ra.y;
                        // b's triangles, one per thread, against the patch
                        for (int base = 0; base < rb.y && !meets; base += kPairThreads) {
                            const int k = base + tid;
                            bool hit = false;
                            bool near = k < rb.y;
                            if (near && P.b.tri_chunk_box) {  // the triangle's chunk box first
                                const float* cb = P.b.tri_chunk_box + 6 * (size_t)((rb.x + k) >> 5);
                                near = box_overlap(__ldg(cb), __ldg(cb + 3), __ldg(cb + 1), __ldg(cb + 4), __ldg(cb + 2),
                                                   __ldg(cb + 5), lo, hi);
                            }
                            if (near) {
                                const uint32_t tb = (uint32_t)(rb.x + k);
                                const float3 b0 = tri_vertex(P.b, tb, 0), b1 = tri_vertex(P.b, tb, 1),
                                             b2 = tri_vertex(P.b, tb, 2);
                                const float3 blo = make_float3(fminf(b0.x, fminf(b1.x, b2.x)), fminf(b0.y, fminf(b1.y, b2.y)),
                                                               fminf(b0.z, fminf(b1.z, b2.z)));
                                const float3 bhi = make_float3(fmaxf(b0.x, fmaxf(b1.x, b2.x)), fmaxf(b0.y, fmaxf(b1.y, b2.y)),
                                                               fmaxf(b0.z, fmaxf(b1.z, b2.z)));
                                if (box_overlap(blo.x, bhi.x, blo.y, bhi.y, blo.z, bhi.z, lo, hi)) {
                                    for (int j = 0; j < nj && !hit; ++j) {
                                        float3 a0, a1, a2;
                                        if (cached) {
                                            const float4 x0 = s_tri[j][0], x1 = s_tri[j][1], x2 = s_tri[j][2];
                                            a0 = make_float3(x0.x, x0.y, x0.z);
                                            a1 = make_float3(x1.x, x1.y, x1.z);
                                            a2 = make_float3(x2.x, x2.y, x2.z);
                                        } else {
                                            const uint32_t ta = listed ? s_list[j] : (uint32_t)(ra.x + j);
                                            a0 = tri_vertex(P.a, ta, 0);
                                            a1 = tri_vertex(P.a, ta, 1);
                                            a2 = tri_vertex(P.a, ta, 2);
                                        }
                                        if (!tri_box_meets(a0, a1, a2, blo, bhi)) continue;
                                        ++tests;
                                        hit = seg_tri_exact(a0, a1, b0, b1, b2, pc) || seg_tri_exact(a1, a2, b0, b1, b2, pc) ||
                                              seg_tri_exact(a2, a0, b0, b1, b2, pc) || seg_tri_exact(b0, b1, a0, a1, a2, pc) ||
                                              seg_tri_exact(b1, b2, a0, a1, a2, pc) || seg_tri_exact(b2, b0, a0, a1, a2, pc);
                                    }
                                }
                            }
                            meets = __syncthreads_or(hit) != 0;
                        }
                    }
                }
            }
            if (tid == 0) {
                if (undecided) {
                    atomicAdd(P.fallback, 1ull);
                } else if (!meets) {
                    const unsigned long long pos = atomicAdd(P.count, 1ull);
                    if (pos < P.cap) P.out[pos] = key;
                }
            }
            __syncthreads();
        }
    }
    flush_counter(&P.ctr->tri_tests, tests);
    flush_counter(&P.ctr->fp32_ambiguous, pc.fp32_ambiguous);
    flush_counter(&P.ctr->fp64_ambiguous, pc.fp64_ambiguous);
}

// Occupied slots -> dense key array (warp-aggregated cursor).  The counter
// counts every occupied slot, so an undersized output is detected.
__global__ void k_compact(const uint64_t* __restrict__ table, uint64_t slots, uint64_t* __restrict__ out,
                          unsigned long long* count, uint64_t cap) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x; base < slots; base += stride) {
        const uint64_t i = base + threadIdx.x;
        const uint64_t key = i < slots ? __ldcs(table + i) : kEmptyKey;
        const bool valid = key != kEmptyKey;
        const unsigned ballot = __ballot_sync(0xFFFFFFFFu, valid);
        if (!ballot) continue;
        const int lane = threadIdx.x & 31;
        unsigned long long wbase = 0;
        if (lane == 0) wbase = atomicAdd(count, (unsigned long long)__popc(ballot));
        wbase = __shfl_sync(0xFFFFFFFFu, wbase, 0);
        if (valid) {
            const unsigned long long pos = wbase + __popc(ballot & ((1u << lane) - 1u));
            if (pos < cap) out[pos] = key;
        }
    }
}

// sorted keys (a << 32 | b) -> pierce_pair {a, b}, in place
__global__ void k_keys_to_pairs(uint64_t* keys, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        keys[i] = (k >> 32) | (k << 32);
    }
}

// pierce_pair {a, b} -> key (a << 32 | b)
__global__ void k_pairs_to_keys(const uint64_t* __restrict__ pairs, uint64_t* __restrict__ keys, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t v = pairs[i];
        keys[i] = (v >> 32) | (v << 32);
    }
}

// =====================================================================
// host side
// =====================================================================


static inline int grid_cap(pierce_ctx* ctx, int64_t n, int block) {
    int64_t blocks = (n + block - 1) / block;
    const int64_t cap = (int64_t)ctx->sm_count * 32;
    if (blocks > cap) blocks = cap;
    return (int)(blocks < 1 ? 1 : blocks);
}

static uint64_t next_pow2(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

int launch_edge_rays(pierce_ctx* ctx, const DevDataset& src, const DevDataset& tgt, int mode, int precision,
                     int swap, int32_t* counts, const int64_t* offsets, uint64_t* keys, uint64_t* table,
                     uint64_t slots, const RayOpts* ro) {
    const int64_t n_rays = (ro && ro->list && ro->bound >= 0) ? ro->bound : src.num_edges;
    if (n_rays == 0) return PIERCE_OK;
    EdgeRayParams P;
    P.src = src;
    P.tgt = tgt;
    P.swap = swap;
    P.counts = counts;
    P.offsets = offsets;
    P.keys = keys;
    P.table = table;
    P.mask = slots ? slots - 1 : 0;
    P.err = ctx->d_err;
    P.ctr = ctx->d_counters;
    P.ray_list = ro ? ro->list : nullptr;
    P.ray_count = ro ? ro->count : nullptr;
    P.ray_cursor = ro ? ro->cursor : nullptr;
    P.amb_queue = ro ? ro->amb_queue : nullptr;
    P.amb_count = ro ? ro->amb_count : nullptr;
    P.amb_cap = ro ? ro->amb_cap : 0;
    P.rays_per_fetch = (ro && ro->rays_per_fetch > 0) ? ro->rays_per_fetch : 32;
    P.short_stack = (ro && ro->short_stack >= 0) ? std::min(ro->short_stack, kShortStack)
                                                  : (P.ray_list ? kCulledShortStack : kShortStack);
    P.packets = (ro && ro->packets && ro->list) ? 1 : 0;
    P.ray_soup = (ro && ro->list) ? ro->soup : nullptr;
    P.ray_bound = n_rays;
    P.shard_count = (ro && ro->shard_count > 1) ? ro->shard_count : 1;
    P.shard_index = (ro && ro->shard_count > 1) ? ro->shard_index : 0;
    // entry nodes hold for the unpartitioned four-wide hierarchy they were found in
    const bool entries = ro && ro->list && ro->soup && ro->entries && tgt.nodes4 && !tgt.part_roots &&
                         !tgt.root_is_leaf && !P.packets;
    P.ray_entry = entries ? ro->entries : nullptr;
    P.entry_group = entries ? std::max(ro->entry_group, 1) : 1;
    if (P.rays_per_fetch % 32 != 0 || P.rays_per_fetch > 1024)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "rays per warp must be a multiple of 32, at most 1024");
    if (precision == PREC_DEFER && !P.amb_queue) precision = PREC_EXACT;
    const int B = 128;
    // per-thread short stacks, then (packets) one (node, mask) stack per warp
    const size_t smem = sizeof(int) * 128 * (size_t)P.short_stack + (P.packets ? sizeof(int2) * 4 * kStackSize : 0);
    dim3 g;
    if (P.ray_list) {
        cudaMemsetAsync(P.ray_cursor, 0, sizeof(unsigned long long), ctx->stream);
        const int64_t want = (n_rays + B - 1) / B;
        g = dim3((unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)ctx->sm_count * 12)));
    } else {
        const int64_t blocks = (src.num_edges + B - 1) / B;
        if (blocks > 0x7FFFFFFF) return set_error(PIERCE_ERR_INVALID_ARGUMENT, "too many edges for one launch");
        g = dim3((unsigned)blocks);
    }
    cudaStream_t st = ctx->stream;
#define PG_LAUNCH(M, PR)                                    \
    do {                                                    \
        if (P.ray_list && P.packets && P.ray_soup) k_edge_rays<M, PR, 2, 1><<<g, B, smem, st>>>(P); \
        else if (P.ray_list && P.packets) k_edge_rays<M, PR, 2, 0><<<g, B, smem, st>>>(P);         \
        else if (P.ray_list && P.ray_soup) k_edge_rays<M, PR, 1, 1><<<g, B, smem, st>>>(P);        \
        else if (P.ray_list) k_edge_rays<M, PR, 1, 0><<<g, B, smem, st>>>(P);                      \
        else k_edge_rays<M, PR, 0, 0><<<g, B, smem, st>>>(P);                                      \
    } while (0)
#define PG_MODES(PR)                                  \
    do {                                              \
        if (mode == MODE_COUNT) PG_LAUNCH(MODE_COUNT, PR); \
        else if (mode == MODE_WRITE) PG_LAUNCH(MODE_WRITE, PR); \
        else PG_LAUNCH(MODE_HASH, PR);                \
    } while (0)
    if (precision == PREC_EXACT) PG_MODES(PREC_EXACT);
    else if (precision == PREC_DEFER) PG_MODES(PREC_DEFER);
    else PG_MODES(PREC_FP32);
#undef PG_MODES
#undef PG_LAUNCH
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "edge ray kernel");
}

int launch_resolve(pierce_ctx* ctx, const DevDataset& src, const DevDataset& tgt, int swap, uint64_t* table,
                   uint64_t slots, const RayOpts* ro, uint64_t* keys_out, unsigned long long* keys_count,
                   uint64_t keys_cap) {
    EdgeRayParams P;
    std::memset(&P, 0, sizeof(P));
    P.src = src;
    P.tgt = tgt;
    P.swap = swap;
    P.table = table;
    P.mask = slots ? slots - 1 : 0;
    P.err = ctx->d_err;
    P.ctr = ctx->d_counters;
    P.amb_queue = ro->amb_queue;
    P.amb_count = ro->amb_count;
    P.amb_cap = ro->amb_cap;
    P.ray_soup = ro->list ? ro->soup : nullptr;
    k_resolve_ambiguous<<<ctx->sm_count * 4, 128, 0, ctx->stream>>>(P, keys_out, keys_count, keys_cap);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "resolve ambiguous tests");
}

int launch_object_active(pierce_ctx* ctx, const DevDataset& src, const DevDataset& tgt, uint8_t* active) {
    if (src.num_objects <= 0) return PIERCE_OK;
    k_object_active<<<(unsigned)((src.num_objects + 127) / 128), 128, 0, ctx->stream>>>(src, tgt, active);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "object activity");
}

int launch_collect_rays(pierce_ctx* ctx, const DevDataset& src, const uint8_t* active, uint32_t* list,
                        unsigned long long* count) {
    cudaMemsetAsync(count, 0, sizeof(unsigned long long), ctx->stream);
    if (src.num_edges > 0) {
        k_collect_rays<<<grid_cap(ctx, (src.num_edges + 7) / 8, 256), 256, 0, ctx->stream>>>(
            src.edge_src, src.num_edges, active, list, count);
        ctx->launches += 1;
    }
    return check_cuda(cudaGetLastError(), "collect rays");
}

int launch_cull(pierce_ctx* ctx, const DevDataset& src, const DevDataset& tgt, uint8_t* active, uint32_t* list,
                unsigned long long* count) {
    if (int s = launch_object_active(ctx, src, tgt, active)) return s;
    return launch_collect_rays(ctx, src, active, list, count);
}

// ---- chunk culling -------------------------------------------------------------
// Consecutive triangles (and consecutive edges) of a mesh lie close together,
// so chunks of kChunk of them get one box: a chunk whose box meets no object
// box of the other side cannot take part in an overlap pair (a triangle or
// edge lies in its chunk's box, and every triangle of the other side lies in
// its object's box).  A warp forms the boxes of 32 chunks, one per lane, and
// every lane then queries the other side's object hierarchy with its box.
constexpr int kChunk = 32;

// Does leaf [first, first + count) of `h` meet [lo, hi]?  A soup of boxes
// (degenerate triangles lo, hi, hi) is tested box by box, a soup of
// triangles by each triangle's box.
__device__ __forceinline__ bool leaf_meets_box(const DevDataset& h, int first, int count, const float3& lo,
                                               const float3& hi) {
    for (int k = 0; k < count; ++k) {
        const int64_t t = (int64_t)first + k;
        const float4 a4 = __ldg(h.soup + 3 * t), b4 = __ldg(h.soup + 3 * t + 1);
        if (h.soup_boxes) {
            if (box_overlap(a4.x, b4.x, a4.y, b4.y, a4.z, b4.z, lo, hi)) return true;
        } else {
            const float4 c4 = __ldg(h.soup + 3 * t + 2);
            if (box_overlap(fminf(a4.x, fminf(b4.x, c4.x)), fmaxf(a4.x, fmaxf(b4.x, c4.x)),
                            fminf(a4.y, fminf(b4.y, c4.y)), fmaxf(a4.y, fmaxf(b4.y, c4.y)),
                            fminf(a4.z, fminf(b4.z, c4.z)), fmaxf(a4.z, fmaxf(b4.z, c4.z)), lo, hi))
                return true;
        }
    }
    return false;
}

// Per-join builds over groups of triangles keep only the groups whose box
// meets a leaf item of `other`, a four-wide hierarchy of the other side:
// object boxes, surviving chunk boxes, or the other side's kept triangles.
// A group that meets none cannot meet the other side's edges, which lie in
// those boxes.
// Partitioned sides (gt2o and obj_part given): a group only meets the other
// side's subtree of its own partition.
__global__ void __launch_bounds__(256) k_group_filter(const float* __restrict__ gbox, int64_t ng, DevDataset other,
                                                      const int32_t* __restrict__ gt2o,
                                                      const int32_t* __restrict__ obj_part,
                                                      uint8_t* __restrict__ flags) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < ng; g += (int64_t)gridDim.x * blockDim.x) {
        const float* b = gbox + 6 * g;
        const float3 lo = make_float3(b[0], b[1], b[2]), hi = make_float3(b[3], b[4], b[5]);
        auto leaf_hit = [&](int first, int count) { return leaf_meets_box(other, first, count, lo, hi); };
        bool keep = true;  // without a hierarchy (a single root leaf) keep everything
        if (gt2o && obj_part && other.part_roots) {
            const int32_t o = __ldg(gt2o + g);
            const int2 r = o >= 0 ? __ldg(other.part_roots + __ldg(obj_part + o)) : make_int2(-1, 0);
            if (!(lo.x <= hi.x)) keep = true;
            else if (r.x >= 0) keep = other.nodes4 ? any_hit4(other.nodes4, r.x, lo, hi, leaf_hit) : true;
            else keep = r.y > 0 && leaf_hit(~r.x, r.y);
        } else if (!other.root_is_leaf && other.nodes4 && lo.x <= hi.x) {
            keep = any_hit4(other.nodes4, 0, lo, hi, leaf_hit);
        } else if (other.num_tris == 0) {
            keep = false;
        }
        flags[g] = keep ? 1 : 0;
    }
}

int launch_group_filter(pierce_ctx* ctx, const float* gbox, int64_t ng, const DevDataset& other,
                        const int32_t* gt2o, const int32_t* obj_part, uint8_t* flags) {
    if (ng <= 0) return PIERCE_OK;
    const int64_t blocks = std::min<int64_t>((ng + 255) / 256, (int64_t)ctx->sm_count * 16);
    k_group_filter<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, ctx->stream>>>(gbox, ng, other, gt2o, obj_part,
                                                                                  flags);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "group filter");
}

// ---- rays from the kept triangles ---------------------------------------------
// A join that builds per-join hierarchies over the triangles that can take
// part in an overlap pair traces the edges of those triangles instead of the
// dataset's edge list: an edge of one side that meets the other side at x is
// an edge of a triangle of its own side that contains x, and the culling
// rounds keep every triangle that contains a point of the other side.  The
// soup holds the kept triangles G at a time (one group per leaf).  A group's
// rays are the edges of its triangles, each segment once per group (an edge
// two triangles of the group share, in either orientation, is listed once;
// an edge shared across groups is traced once per group, which only repeats
// work: pairs are de-duplicated).  With a filter hierarchy only the groups
// whose box meets one of its leaf items are listed.  List entry (t << 2) | k:
// edge k of soup triangle t.

__device__ __forceinline__ bool same_point(const float4& a, const float4& b) {
    return a.x == b.x && a.y == b.y && a.z == b.z;
}

// Edge k (0: v0 v1, 1: v1 v2, 2: v2 v0) of soup triangle t repeats an edge
// listed before it in its group: an edge of triangles first .. t - 1, or
// edges 0 .. k - 1 of t.
__device__ bool edge_listed_before(const float4* __restrict__ soup, int64_t first, int64_t t, int k, const float4& p,
                                   const float4& q) {
    for (int64_t u = first; u <= t; ++u) {
        const float4 w[3] = {__ldg(soup + 3 * u), __ldg(soup + 3 * u + 1), __ldg(soup + 3 * u + 2)};
        const int kmax = u < t ? 3 : k;
        for (int j = 0; j < kmax; ++j) {
            const float4& a = w[j];
            const float4& b = w[j == 2 ? 0 : j + 1];
            if ((same_point(a, p) && same_point(b, q)) || (same_point(a, q) && same_point(b, p))) return true;
        }
    }
    return false;
}

// Does the box [lo, hi] of a group of object `obj` meet a leaf item of the
// four-wide hierarchy `other` (within the object's partition)?
__device__ bool group_meets(const DevDataset& other, const int32_t* __restrict__ obj_part, int32_t obj,
                            const float3& lo, const float3& hi) {
    if (!(lo.x <= hi.x && lo.y <= hi.y && lo.z <= hi.z)) return true;  // NaN coordinates: keep
    auto leaf_hit = [&](int first, int count) { return leaf_meets_box(other, first, count, lo, hi); };
    if (obj_part && other.part_roots) {
        const int2 r = __ldg(other.part_roots + __ldg(obj_part + obj));
        if (r.x >= 0) return other.nodes4 ? any_hit4(other.nodes4, r.x, lo, hi, leaf_hit) : true;
        return r.y > 0 && leaf_hit(~r.x, r.y);
    }
    if (other.num_tris == 0) return false;
    if (other.root_is_leaf) return leaf_hit(0, other.root_leaf_count);
    return other.nodes4 ? any_hit4(other.nodes4, 0, lo, hi, leaf_hit) : true;
}

// Unique edges of a group of up to GMAX soup triangles [first, last): bit
// 3 t + k of the result is set when edge k of triangle first + t is the first
// occurrence of its segment in the group.  The group's vertices are loaded
// once; each gets the id of the first vertex with the same coordinates, and
// edges compare as unordered id pairs.
// Shard of a segment among n shards, from its endpoints alone: the same
// segment listed by any triangle, in either orientation, lands in one shard
// (coordinates in lexicographic order, -0 taken as +0, hashed).
__device__ __forceinline__ int seg_shard(const float4& p, const float4& q, int n) {
    const bool swap = q.x < p.x || (q.x == p.x && (q.y < p.y || (q.y == p.y && q.z < p.z)));
    const float4& a = swap ? q : p;
    const float4& b = swap ? p : q;
    auto bits = [](float f) { return (uint64_t)__float_as_uint(__fadd_rn(f, 0.0f)); };
    uint64_t h = fmix64((bits(a.x) << 32) | bits(a.y));
    h = fmix64(h ^ ((bits(a.z) << 32) | bits(b.x)));
    h = fmix64(h ^ ((bits(b.y) << 32) | bits(b.z)));
    return (int)(h % (uint64_t)n);
}

template <int GMAX>
__device__ __forceinline__ uint32_t group_unique_edges(const float4* __restrict__ soup, int64_t first, int64_t last,
                                                       float3& lo, float3& hi, int shard_index, int shard_count) {
    static_assert(3 * GMAX <= 16, "vertex ids are packed in 4 bits");
    const int nv = 3 * (int)(last - first);
    const float4* v = soup + 3 * first;
    lo = make_float3(3.4e38f, 3.4e38f, 3.4e38f);
    hi = make_float3(-3.4e38f, -3.4e38f, -3.4e38f);
    // vertex i's id: the first vertex of the group with its coordinates
    // (4 bits each; the vertices are read again rather than kept)
    uint64_t ids = 0;
    for (int i = 0; i < nv; ++i) {
        const float4 a = __ldg(v + i);
        lo.x = fminf(lo.x, a.x); lo.y = fminf(lo.y, a.y); lo.z = fminf(lo.z, a.z);
        hi.x = fmaxf(hi.x, a.x); hi.y = fmaxf(hi.y, a.y); hi.z = fmaxf(hi.z, a.z);
        uint64_t c = (uint64_t)i;
        for (int j = 0; j < i; ++j)
            if (same_point(__ldg(v + j), a)) {
                c = (ids >> (4 * j)) & 15u;
                break;
            }
        ids |= c << (4 * i);
    }
    // edge e = 3 t + k joins vertices 3 t + k and 3 t + (k + 1) % 3; its key is
    // the unordered id pair (8 bits each, packed in two words)
    uint64_t keys[2] = {0, 0};
    uint32_t mask = 0;
    for (int e = 0; e < nv; ++e) {
        const int t = e / 3, k = e - 3 * t;
        const int ia = 3 * t + k, ib = 3 * t + (k == 2 ? 0 : k + 1);
        const uint32_t a = (uint32_t)(ids >> (4 * ia)) & 15u, b = (uint32_t)(ids >> (4 * ib)) & 15u;
        const uint64_t key = a < b ? a * 16 + b : b * 16 + a;
        bool dup = false;
        for (int f = 0; f < e && !dup; ++f) dup = ((keys[f >> 3] >> (8 * (f & 7))) & 255u) == key;
        if (e < 8) keys[0] |= key << (8 * e);
        else keys[1] |= key << (8 * (e - 8));
        if (!dup && shard_count > 1) dup = seg_shard(__ldg(v + ia), __ldg(v + ib), shard_count) != shard_index;
        if (!dup) mask |= 1u << e;
    }
    return mask;
}

// Entry node of a group's walks in the four-wide hierarchy `tgt` (not
// partitioned, root not a leaf): from the root, descend while exactly one
// child box meets the group's box [lo, hi] and that child is internal.
// Every leaf whose box meets the group's box lies under the node returned,
// so a walk of any segment inside that box that starts there reaches the
// same leaves, in the same order, as one that starts at the root.
__device__ __forceinline__ int32_t group_entry(const Node4* __restrict__ nodes4, const float3& lo, const float3& hi) {
    if (!(lo.x <= hi.x && lo.y <= hi.y && lo.z <= hi.z)) return 0;  // NaN coordinates: the root
    int32_t node = 0;
    for (int depth = 0; depth < 64; ++depth) {
        const Node4* nd = nodes4 + node;
        const float4 lx = __ldg(&nd->lox), hx = __ldg(&nd->hix), ly = __ldg(&nd->loy), hy = __ldg(&nd->hiy);
        const float4 lz = __ldg(&nd->loz), hz = __ldg(&nd->hiz);
        const int4 ch = __ldg(&nd->ch);
        const bool h[4] = {box_overlap(lx.x, hx.x, ly.x, hy.x, lz.x, hz.x, lo, hi),
                           box_overlap(lx.y, hx.y, ly.y, hy.y, lz.y, hz.y, lo, hi),
                           box_overlap(lx.z, hx.z, ly.z, hy.z, lz.z, hz.z, lo, hi),
                           box_overlap(lx.w, hx.w, ly.w, hy.w, lz.w, hz.w, lo, hi)};
        const int c[4] = {ch.x, ch.y, ch.z, ch.w};
        int hits = 0, only = -1;
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (h[j]) {
                ++hits;
                only = c[j];
            }
        if (hits != 1 || only < 0) return node;
        node = only;
    }
    return node;
}

// One thread per group; whole blocks step through the groups together so
// that a warp reserves its list range with one atomicAdd.  GMAX: the group
// size the kernel keeps in registers (G <= GMAX); larger groups take the
// loop over the soup (edge_listed_before).
template <int GMAX>
__global__ void __launch_bounds__(256) k_soup_rays(const float4* __restrict__ soup, int64_t n_tris, int G,
                                                   DevDataset filter, int use_filter,
                                                   const int32_t* __restrict__ obj_part, uint32_t* __restrict__ list,
                                                   unsigned long long* __restrict__ count, int shard_index,
                                                   int shard_count, const Node4* __restrict__ entry_nodes4,
                                                   int32_t* __restrict__ entries) {
    const int64_t n_groups = (n_tris + G - 1) / G;
    // a split join lists only the segments of its shard (seg_shard)
    auto mine = [&](const float4& p, const float4& q) {
        return shard_count <= 1 || seg_shard(p, q, shard_count) == shard_index;
    };
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n_groups; base += stride) {
        const int64_t g = base + threadIdx.x;
        const int64_t first = g * G;
        const int64_t last = min(first + (int64_t)G, n_tris);
        bool keep = g < n_groups;
        uint32_t mask = 0;
        float3 lo = make_float3(0, 0, 0), hi = make_float3(0, 0, 0);
        if (keep) {
            if constexpr (GMAX > 0) {
                mask = group_unique_edges<GMAX>(soup, first, last, lo, hi, shard_index, shard_count);
            } else {
                lo = make_float3(3.4e38f, 3.4e38f, 3.4e38f);
                hi = make_float3(-3.4e38f, -3.4e38f, -3.4e38f);
                for (int64_t t = first; t < last; ++t)
                    for (int v = 0; v < 3; ++v) {
                        const float4 a = __ldg(soup + 3 * t + v);
                        lo.x = fminf(lo.x, a.x); lo.y = fminf(lo.y, a.y); lo.z = fminf(lo.z, a.z);
                        hi.x = fmaxf(hi.x, a.x); hi.y = fmaxf(hi.y, a.y); hi.z = fmaxf(hi.z, a.z);
                    }
            }
        }
        if (keep && use_filter) {
            const int32_t obj0 = __float_as_int(__ldg(&soup[3 * first].w));
            bool one_part = true;  // a group spanning partitions is kept
            if (obj_part && filter.part_roots) {
                const int32_t p0 = __ldg(obj_part + obj0);
                for (int64_t t = first + 1; t < last; ++t)
                    one_part = one_part && __ldg(obj_part + __float_as_int(__ldg(&soup[3 * t].w))) == p0;
            }
            keep = !one_part || group_meets(filter, obj_part, obj0, lo, hi);
        }
        // the walks of a listed group's segments start at its entry node
        if (keep && entries) entries[g] = group_entry(entry_nodes4, lo, hi);
        int n = 0;
        if (keep) {
            if constexpr (GMAX > 0) {
                n = __popc(mask);
            } else {
                for (int64_t t = first; t < last; ++t)
                    for (int k = 0; k < 3; ++k) {
                        const float4 p = __ldg(soup + 3 * t + k), q = __ldg(soup + 3 * t + (k == 2 ? 0 : k + 1));
                        if (!edge_listed_before(soup, first, t, k, p, q) && mine(p, q)) ++n;
                    }
            }
        }
        int incl = n;
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xFFFFFFFFu, incl, off);
            if (lane >= off) incl += y;
        }
        const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
        unsigned long long wbase = 0;
        if (lane == 31 && total) wbase = atomicAdd(count, (unsigned long long)total);
        wbase = __shfl_sync(0xFFFFFFFFu, wbase, 31);
        unsigned long long pos = wbase + (unsigned long long)(incl - n);
        if (n) {
            if constexpr (GMAX > 0) {
                for (uint32_t m = mask; m; m &= m - 1) {
                    const int e = __ffs(m) - 1;
                    list[pos++] = (uint32_t)(((first + e / 3) << 2) | (e % 3));
                }
            } else {
                for (int64_t t = first; t < last; ++t)
                    for (int k = 0; k < 3; ++k) {
                        const float4 p = __ldg(soup + 3 * t + k), q = __ldg(soup + 3 * t + (k == 2 ? 0 : k + 1));
                        if (!edge_listed_before(soup, first, t, k, p, q) && mine(p, q))
                            list[pos++] = (uint32_t)((t << 2) | k);
                    }
            }
        }
    }
}

// Pair-count bound for output sizing: every step-th group of G source soup
// triangles against the target's four-wide per-join hierarchy, counting the
// target triangles whose box meets the group's box (a run of one target
// object counts once).  Every overlap pair has a kept source group whose box
// meets a kept target triangle of the pair's target object, so step x this
// count estimates an upper bound on the join's pairs.
__global__ void __launch_bounds__(256) k_group_incidences(const float4* __restrict__ soup, int64_t n_tris, int G,
                                                          int step, DevDataset tgt, unsigned long long* count) {
    const int64_t n_groups = (n_tris + G - 1) / G;
    unsigned long long local = 0;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s * step < n_groups;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t first = s * step * G, last = min(first + (int64_t)G, n_tris);
        float3 lo = make_float3(3.4e38f, 3.4e38f, 3.4e38f), hi = make_float3(-3.4e38f, -3.4e38f, -3.4e38f);
        for (int64_t t = first; t < last; ++t)
            for (int v = 0; v < 3; ++v) {
                const float4 a = __ldg(soup + 3 * t + v);
                lo.x = fminf(lo.x, a.x); lo.y = fminf(lo.y, a.y); lo.z = fminf(lo.z, a.z);
                hi.x = fmaxf(hi.x, a.x); hi.y = fmaxf(hi.y, a.y); hi.z = fmaxf(hi.z, a.z);
            }
        int32_t last_obj = -1;
        auto visit = [&](int lfirst, int lcount) {
            for (int k = 0; k < lcount; ++k) {
                const int64_t t = (int64_t)lfirst + k;
                const float4 a4 = __ldg(tgt.soup + 3 * t), b4 = __ldg(tgt.soup + 3 * t + 1),
                             c4 = __ldg(tgt.soup + 3 * t + 2);
                const int32_t obj = __float_as_int(a4.w);
                if (obj == last_obj) continue;
                if (box_overlap(fminf(a4.x, fminf(b4.x, c4.x)), fmaxf(a4.x, fmaxf(b4.x, c4.x)),
                                fminf(a4.y, fminf(b4.y, c4.y)), fmaxf(a4.y, fmaxf(b4.y, c4.y)),
                                fminf(a4.z, fminf(b4.z, c4.z)), fmaxf(a4.z, fmaxf(b4.z, c4.z)), lo, hi)) {
                    last_obj = obj;
                    ++local;
                }
            }
            return false;  // visit every leaf the box meets
        };
        if (tgt.root_is_leaf) visit(0, tgt.root_leaf_count);
        else if (tgt.nodes4) any_hit4(tgt.nodes4, 0, lo, hi, visit);
    }
    flush_counter(count, local);
}

int launch_group_incidences(pierce_ctx* ctx, const float4* soup, int64_t n_tris, int G, int step,
                            const DevDataset& tgt, unsigned long long* count) {
    cudaMemsetAsync(count, 0, sizeof(unsigned long long), ctx->stream);
    if (n_tris <= 0 || tgt.num_tris <= 0 || (!tgt.root_is_leaf && !tgt.nodes4)) return PIERCE_OK;
    const int64_t samples = ((n_tris + G - 1) / G + step - 1) / step;
    const int64_t blocks = std::min<int64_t>((samples + 255) / 256, (int64_t)ctx->sm_count * 8);
    k_group_incidences<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, ctx->stream>>>(soup, n_tris, G, step, tgt,
                                                                                          count);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "group incidences");
}

int launch_soup_rays(pierce_ctx* ctx, const float4* soup, int64_t n_tris, int G, const DevDataset* filter,
                     const int32_t* obj_part, uint32_t* list, unsigned long long* count, int shard_index,
                     int shard_count, const Node4* entry_nodes4, int32_t* entries) {
    if (!entry_nodes4) entries = nullptr;
    cudaMemsetAsync(count, 0, sizeof(unsigned long long), ctx->stream);
    if (n_tris <= 0) return check_cuda(cudaGetLastError(), "rays from triangles");
    if (n_tris >= (int64_t(1) << 30))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "rays from triangles: at most 2^30 - 1 triangles");
    const int64_t n_groups = (n_tris + G - 1) / G;
    const int64_t blocks = std::min<int64_t>((n_groups + 255) / 256, (int64_t)ctx->sm_count * 16);
    const unsigned grid = (unsigned)std::max<int64_t>(blocks, 1);
    const DevDataset f = filter ? *filter : DevDataset{};
    if (G <= 1)
        k_soup_rays<1><<<grid, 256, 0, ctx->stream>>>(soup, n_tris, G, f, filter ? 1 : 0, obj_part, list, count,
                                                             shard_index, shard_count, entry_nodes4, entries);
    else if (G <= 2)
        k_soup_rays<2><<<grid, 256, 0, ctx->stream>>>(soup, n_tris, G, f, filter ? 1 : 0, obj_part, list, count,
                                                             shard_index, shard_count, entry_nodes4, entries);
    else if (G <= 4)
        k_soup_rays<4><<<grid, 256, 0, ctx->stream>>>(soup, n_tris, G, f, filter ? 1 : 0, obj_part, list, count,
                                                             shard_index, shard_count, entry_nodes4, entries);
    else
        k_soup_rays<0><<<grid, 256, 0, ctx->stream>>>(soup, n_tris, G, f, filter ? 1 : 0, obj_part, list, count,
                                                             shard_index, shard_count, entry_nodes4, entries);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "rays from triangles");
}

// Does [lo, hi] meet an item of `objs` within partition `part`?  Items are
// the boxes of a box hierarchy (object or chunk boxes as degenerate
// triangles) or the triangles of a per-join hierarchy (by their boxes).
__device__ bool meets_any_object(const DevDataset& objs, int32_t part, const float3& lo, const float3& hi) {
    auto leaf_hit = [&](int first, int count) { return leaf_meets_box(objs, first, count, lo, hi); };
    int node;
    if (objs.part_roots) {
        const int2 r = __ldg(objs.part_roots + part);
        if (r.x < 0) return leaf_hit(~r.x, r.y);
        node = r.x;
    } else if (objs.root_is_leaf) {
        return leaf_hit(0, objs.root_leaf_count);
    } else {
        node = 0;
    }
    if (objs.nodes4) return any_hit4(objs.nodes4, node, lo, hi, leaf_hit);
    int stack[kStackSize];
    int sp = 0;
    for (;;) {
        const Node* nd = objs.nodes + node;
        const float4 bx = __ldg(&nd->bx), by = __ldg(&nd->by), bz = __ldg(&nd->bz);
        const int4 ch = __ldg(&nd->ch);
        bool h0 = box_overlap(bx.x, bx.y, by.x, by.y, bz.x, bz.y, lo, hi);
        bool h1 = box_overlap(bx.z, bx.w, by.z, by.w, bz.z, bz.w, lo, hi);
        if (h0 && ch.x < 0) {
            if (leaf_hit(~ch.x, ch.z & 0xFF)) return true;
            h0 = false;
        }
        if (h1 && ch.y < 0) {
            if (leaf_hit(~ch.y, (ch.z >> 8) & 0xFF)) return true;
            h1 = false;
        }
        if (h0 && h1) {
            if (sp >= kStackSize) return true;  // cannot happen for an LBVH; stay conservative
            stack[sp++] = ch.y;
            node = ch.x;
        } else if (h0) {
            node = ch.x;
        } else if (h1) {
            node = ch.y;
        } else {
            if (sp == 0) return false;
            node = stack[--sp];
        }
    }
}

// Per chunk of triangles (EDGES = false) or edges (EDGES = true) of `src`:
// 1 when its box, over the items of active objects, meets an object box of
// the other side.  A chunk whose items span partitions stays active.
template <bool EDGES>
__global__ void __launch_bounds__(128) k_chunk_active(const float* __restrict__ verts,
                                                      const uint32_t* __restrict__ idx,
                                                      const int32_t* __restrict__ t2o, const float4* __restrict__ edges,
                                                      const int32_t* __restrict__ edge_src, int64_t n,
                                                      const uint8_t* __restrict__ obj_active,
                                                      const int32_t* __restrict__ obj_part, DevDataset objs,
                                                      uint8_t* __restrict__ chunk_active,
                                                      float* __restrict__ chunk_box,
                                                      const float* __restrict__ pre_box, bool items_contiguous) {
    const int lane = threadIdx.x & 31;
    const int64_t n_chunks = (n + kChunk - 1) / kChunk;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t c0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; c0 < n_chunks;
         c0 += warps * 32) {
        float3 mylo = make_float3(0, 0, 0), myhi = make_float3(0, 0, 0);
        bool myany = false, mymixed = false;
        int32_t mypart = 0;
        if (pre_box) {
            // the dataset's own chunk boxes; with objects stored contiguously
            // a chunk inside one inactive object is skipped outright
            if (c0 + lane < n_chunks) {
                const int64_t i0 = (c0 + lane) * kChunk, i1 = min(i0 + kChunk, n) - 1;
                const int32_t* io = EDGES ? edge_src : t2o;
                bool dead = false;
                if (items_contiguous) {
                    const int32_t o0 = __ldg(io + i0), o1 = __ldg(io + i1);
                    dead = o0 == o1 && (o0 < 0 || __ldg(obj_active + o0) == 0);
                }
                if (!dead) {
                    const float* b = pre_box + 6 * (c0 + lane);
                    mylo = make_float3(__ldg(b), __ldg(b + 1), __ldg(b + 2));
                    myhi = make_float3(__ldg(b + 3), __ldg(b + 4), __ldg(b + 5));
                    myany = mylo.x <= myhi.x;
                }
            }
        }
        for (int j = 0; j < 32 && !pre_box; ++j) {
            const int64_t c = c0 + j;
            if (c >= n_chunks) break;
            const int64_t i = c * kChunk + lane;
            bool valid = i < n;
            int32_t obj = -1;
            float3 lo = make_float3(3.4e38f, 3.4e38f, 3.4e38f), hi = make_float3(-3.4e38f, -3.4e38f, -3.4e38f);
            if (valid) {
                obj = EDGES ? __ldg(edge_src + i) : __ldg(t2o + i);
                valid = obj >= 0 && __ldg(obj_active + obj) != 0;
            }
            if (valid) {
                if (EDGES) {
                    const float4 a = __ldg(edges + 2 * i), b = __ldg(edges + 2 * i + 1);
                    lo = make_float3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z));
                    hi = make_float3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z));
                } else {
                    for (int v = 0; v < 3; ++v) {
                        const uint32_t vi = __ldg(idx + 3 * i + v);
                        const float x = __ldg(verts + 3 * (size_t)vi), y = __ldg(verts + 3 * (size_t)vi + 1),
                                    z = __ldg(verts + 3 * (size_t)vi + 2);
                        lo = make_float3(fminf(lo.x, x), fminf(lo.y, y), fminf(lo.z, z));
                        hi = make_float3(fmaxf(hi.x, x), fmaxf(hi.y, y), fmaxf(hi.z, z));
                    }
                }
            }
            const unsigned vmask = __ballot_sync(0xFFFFFFFFu, valid);
            int32_t part = (valid && obj_part) ? __ldg(obj_part + obj) : 0;
            const int leader = vmask ? __ffs(vmask) - 1 : 0;
            const int32_t p0 = __shfl_sync(0xFFFFFFFFu, part, leader);
            const bool mixed = __any_sync(0xFFFFFFFFu, valid && part != p0);
            for (int off = 16; off > 0; off >>= 1) {
                lo.x = fminf(lo.x, __shfl_xor_sync(0xFFFFFFFFu, lo.x, off));
                lo.y = fminf(lo.y, __shfl_xor_sync(0xFFFFFFFFu, lo.y, off));
                lo.z = fminf(lo.z, __shfl_xor_sync(0xFFFFFFFFu, lo.z, off));
                hi.x = fmaxf(hi.x, __shfl_xor_sync(0xFFFFFFFFu, hi.x, off));
                hi.y = fmaxf(hi.y, __shfl_xor_sync(0xFFFFFFFFu, hi.y, off));
                hi.z = fmaxf(hi.z, __shfl_xor_sync(0xFFFFFFFFu, hi.z, off));
            }
            if (lane == j) {
                mylo = lo;
                myhi = hi;
                myany = vmask != 0;
                mymixed = mixed;
                mypart = p0;
            }
        }
        const int64_t c = c0 + lane;
        if (c < n_chunks) {
            bool act = false;
            if (myany) act = mymixed || meets_any_object(objs, mypart, mylo, myhi);
            chunk_active[c] = act ? 1 : 0;
            if (chunk_box) {  // (lo, hi) as two points: the pseudo-triangle (lo, hi, hi) of the chunk
                float* b = chunk_box + 6 * c;
                b[0] = mylo.x;
                b[1] = mylo.y;
                b[2] = mylo.z;
                b[3] = myhi.x;
                b[4] = myhi.y;
                b[5] = myhi.z;
            }
        }
    }
}

int launch_flag_list(pierce_ctx* ctx, const uint8_t* flags, int64_t n, uint32_t* list, unsigned long long* count) {
    cudaMemsetAsync(count, 0, sizeof(unsigned long long), ctx->stream);
    if (n <= 0) return PIERCE_OK;
    return select_flagged(ctx, flags, n, list, count);  // in index order: deterministic lists
}

// Active chunks -> item list: list[32 k + j] = item j of the k-th listed
// chunk.  A partial final chunk repeats its first item in the unused
// positions (a repeated triangle or ray only repeats hits, which the
// de-duplication removes).  Items of inactive objects inside active chunks
// stay in: they cannot produce pairs, only work.
__global__ void __launch_bounds__(256) k_expand_chunks(const uint32_t* __restrict__ chunk_list,
                                                       const unsigned long long* __restrict__ chunk_count, int64_t n,
                                                       uint32_t* __restrict__ list, unsigned long long* count) {
    const int64_t total = (int64_t)*chunk_count * kChunk;
    if (blockIdx.x == 0 && threadIdx.x == 0) *count = (unsigned long long)total;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = chunk_list[i / kChunk];
        int64_t item = c * kChunk + (i % kChunk);
        if (item >= n) item = c * kChunk;
        list[i] = (uint32_t)item;
    }
}

int launch_chunk_cull(pierce_ctx* ctx, bool edges, const float* verts, const uint32_t* idx, const int32_t* t2o,
                      const DevDataset& src, const uint8_t* obj_active, const DevDataset& objs,
                      uint8_t* chunk_active, uint32_t* list, unsigned long long* count, float* chunk_box,
                      uint32_t* chunk_list, unsigned long long* chunk_count) {
    cudaMemsetAsync(count, 0, sizeof(unsigned long long), ctx->stream);
    const int64_t n = edges ? src.num_edges : src.num_tris;
    if (n <= 0) return PIERCE_OK;
    const int64_t n_chunks = (n + kChunk - 1) / kChunk;
    const int64_t warps = (n_chunks + 31) / 32;
    const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((warps + 3) / 4,
                                                                             (int64_t)ctx->sm_count * 32));
    // unpartitioned datasets read their stored chunk boxes
    const float* pre = src.obj_part ? nullptr : (edges ? src.edge_chunk_box : src.tri_chunk_box);
    // items grouped by object: triangles of a dataset with contiguous objects,
    // edges when the dataset's edges are grouped by source object
    const bool grouped_items = edges ? src.edges_grouped != 0 : src.obj_range != nullptr;
    if (edges)
        k_chunk_active<true><<<blocks, 128, 0, ctx->stream>>>(verts, idx, t2o, src.edges, src.edge_src, n, obj_active,
                                                              src.obj_part, objs, chunk_active, chunk_box, pre, grouped_items);
    else
        k_chunk_active<false><<<blocks, 128, 0, ctx->stream>>>(verts, idx, t2o, src.edges, src.edge_src, n,
                                                               obj_active, src.obj_part, objs, chunk_active,
                                                               chunk_box, pre, grouped_items);
    if (int s = launch_flag_list(ctx, chunk_active, n_chunks, chunk_list, chunk_count)) return s;
    k_expand_chunks<<<grid_cap(ctx, n_chunks * kChunk, 256), 256, 0, ctx->stream>>>(chunk_list, chunk_count, n, list,
                                                                                    count);
    ctx->launches += 2;
    return check_cuda(cudaGetLastError(), "chunk culling");
}

// Triangles of active objects -> compacted list.
__global__ void __launch_bounds__(256) k_collect_tris(const int32_t* __restrict__ t2o, int64_t nt,
                                                      const uint8_t* __restrict__ active, uint32_t* __restrict__ list,
                                                      unsigned long long* count) {
    compact_tiles<8>(nt, [&](int64_t t) {
        const int32_t o = t2o[t];
        return o >= 0 && (!active || active[o] != 0);
    }, list, count);
}

// Object boxes as degenerate triangles (lo, hi, hi): their bounding boxes
// are exactly the object boxes, so the triangle LBVH builder indexes them.
__global__ void k_object_pseudo_tris(int32_t n, uint32_t* idx, int32_t* t2o) {
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x) {
        idx[3 * o] = (uint32_t)(2 * o);
        idx[3 * o + 1] = (uint32_t)(2 * o + 1);
        idx[3 * o + 2] = (uint32_t)(2 * o + 1);
        t2o[o] = (int32_t)o;
    }
}

int launch_collect_tris(pierce_ctx* ctx, const int32_t* t2o, int64_t nt, const uint8_t* active, uint32_t* list,
                        unsigned long long* count) {
    cudaMemsetAsync(count, 0, sizeof(unsigned long long), ctx->stream);
    if (nt > 0) {
        k_collect_tris<<<grid_cap(ctx, (nt + 7) / 8, 256), 256, 0, ctx->stream>>>(t2o, nt, active, list, count);
        ctx->launches += 1;
    }
    return check_cuda(cudaGetLastError(), "collect triangles");
}

int launch_object_pseudo_tris(pierce_ctx* ctx, int32_t n, uint32_t* idx, int32_t* t2o) {
    if (n <= 0) return PIERCE_OK;
    k_object_pseudo_tris<<<grid_cap(ctx, n, 256), 256, 0, ctx->stream>>>(n, idx, t2o);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "object pseudo triangles");
}

int launch_parity(pierce_ctx* ctx, const DevDataset& src, const DevDataset& tgt, int swap, uint64_t* table,
                  uint32_t* parity, uint64_t slots, int64_t src_lo, int64_t src_hi) {
    if (src_hi < 0) src_hi = src.num_objects;
    src_lo = std::max<int64_t>(src_lo, 0);
    src_hi = std::min<int64_t>(src_hi, src.num_objects);
    if (src_hi <= src_lo) return PIERCE_OK;
    ParityParams P;
    P.src = src;
    P.tgt = tgt;
    P.src_lo = src_lo;
    P.src_hi = src_hi;
    P.swap = swap;
    P.table = table;
    P.parity = parity;
    P.mask = slots - 1;
    P.err = ctx->d_err;
    P.ctr = ctx->d_counters;
    const int B = 128;
    k_parity<<<(unsigned)((src_hi - src_lo + B - 1) / B), B, 0, ctx->stream>>>(P);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "parity kernel");
}

__global__ void k_fill_u32_j(uint32_t* p, uint32_t value, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = value;
}

// ---- column grid over object boxes ---------------------------------------
// Parity candidates are the target objects whose box contains the query
// point in x and y and reaches above it.  A uniform grid over the xy plane
// lists, per cell, every object whose box covers the cell in x and y, so a
// query reads one cell's list instead of walking a hierarchy with a column
// that is unbounded above.  About one object per cell on average.


__device__ __forceinline__ void grid_cell_range(const float* b, int nx, int ny, float lo, float hi, int axis,
                                                int& c0, int& c1) {
    const float o = b[axis], e = b[2 + axis] - b[axis];
    const int n = axis ? ny : nx;
    const float inv = e > 0.0f ? (float)n / e : 0.0f;
    c0 = min(max((int)floorf((lo - o) * inv), 0), n - 1);
    c1 = min(max((int)floorf((hi - o) * inv), 0), n - 1);
}

__global__ void k_grid_bounds(const float* __restrict__ obj_box, int32_t n, uint32_t* ob) {
    float lo[2] = {3.4e38f, 3.4e38f}, hi[2] = {-3.4e38f, -3.4e38f};
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x) {
        const float* b = obj_box + 6 * o;
        if (!(b[0] <= b[3])) continue;  // object without triangles
        lo[0] = fminf(lo[0], b[0]); lo[1] = fminf(lo[1], b[1]);
        hi[0] = fmaxf(hi[0], b[3]); hi[1] = fmaxf(hi[1], b[4]);
    }
    for (int k = 0; k < 2; ++k)
        for (int off = 16; off > 0; off >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xFFFFFFFFu, lo[k], off));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xFFFFFFFFu, hi[k], off));
        }
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 2; ++k) {
            const uint32_t ul = __float_as_uint(lo[k]), uh = __float_as_uint(hi[k]);
            atomicMin(ob + k, (ul & 0x80000000u) ? ~ul : (ul | 0x80000000u));
            atomicMax(ob + 2 + k, (uh & 0x80000000u) ? ~uh : (uh | 0x80000000u));
        }
}

__global__ void k_grid_decode(const uint32_t* ob, float* b) {
    const int k = threadIdx.x;
    if (k < 4) {
        const uint32_t u = ob[k];
        float v = __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
        if (!(v == v) || fabsf(v) > 3.0e38f) v = 0.0f;  // no object: empty grid at the origin
        b[k] = v;
    }
}

// MODE 0: count covered cells per cell; MODE 1: write object ids.
template <int MODE>
__global__ void k_grid_fill(const float* __restrict__ obj_box, int32_t n, const float* __restrict__ b, int nx, int ny,
                            int32_t* __restrict__ counts, const int32_t* __restrict__ offsets,
                            int32_t* __restrict__ cursor, int32_t* __restrict__ entries) {
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x) {
        const float* ob = obj_box + 6 * o;
        if (!(ob[0] <= ob[3])) continue;
        int x0, x1, y0, y1;
        grid_cell_range(b, nx, ny, ob[0], ob[3], 0, x0, x1);
        grid_cell_range(b, nx, ny, ob[1], ob[4], 1, y0, y1);
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) {
                const int c = y * nx + x;
                if (MODE == 0) atomicAdd(counts + c, 1);
                else entries[offsets[c] + atomicAdd(cursor + c, 1)] = (int32_t)o;
            }
    }
}

// Parity by object pairs: a warp per source object walks the target's
// object hierarchy with the +Z ray of the object's first vertex (candidate
// target objects: box contains the point in x, y and reaches above it) and
// counts, across its lanes, the crossings of every triangle of each
// candidate (the object's contiguous triangle range).  Odd counts go to the
// parity table.  Needs no triangle hierarchy, so the per-join hierarchies
// can drop triangles far from the other side.
struct ParityObjParams {
    DevDataset src;   // first vertices, partitions
    int64_t src_lo, src_hi;  // source objects [src_lo, src_hi) cast rays (a shard)
    ColumnGrid grid;  // the target's column grid (nx == 0: use the object hierarchy)
    DevDataset objs;  // the target's object hierarchy
    DevDataset tgt;   // the target's triangles (verts, idx, obj_range)
    int swap;
    uint64_t* table;
    uint32_t* parity;
    uint64_t mask;
    uint32_t* err;
    DevCounters* ctr;
    // k_parity_objects<true> (diagnostics) writes, instead of table entries,
    // per source object s: the targets its ray crosses an odd number of times
    // with their crossing counts (slots s * track_k ..., in candidate order),
    // the number of targets it crosses at all, and the odd targets that found
    // no slot
    int32_t track_k;
    int32_t* track_ids;
    uint32_t* track_hits;
    uint32_t* track_crossed;
    uint32_t* track_overflow;
};

template <bool TRACK>
__global__ void __launch_bounds__(128) k_parity_objects(ParityObjParams P) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    uint32_t n_nodes = 0, n_tests = 0, n_rays = 0;
    PredCounters pc{0, 0};
    for (int64_t s = P.src_lo + (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); s < P.src_hi;
         s += warps) {
        const float4 fv = __ldg(P.src.first_vertex + s);
        if (fv.w != 0.0f) continue;  // object without triangles (warp-uniform)
        ++n_rays;
        const float3 p = make_float3(fv.x, fv.y, fv.z);
        uint32_t n_crossed = 0, n_odd = 0;  // TRACK: lane 0's tallies of this source
        auto candidate = [&](int32_t t) {
            const int2 r = __ldg(P.tgt.obj_range + t);
            uint32_t crossings = 0;
            uint32_t ncross = 0;  // TRACK: this lane's crossings
            auto test = [&](int64_t tri) {
                const uint32_t i0 = __ldg(P.tgt.idx + 3 * tri), i1 = __ldg(P.tgt.idx + 3 * tri + 1),
                               i2 = __ldg(P.tgt.idx + 3 * tri + 2);
                const float3 a = make_float3(__ldg(P.tgt.verts + 3 * (size_t)i0), __ldg(P.tgt.verts + 3 * (size_t)i0 + 1),
                                             __ldg(P.tgt.verts + 3 * (size_t)i0 + 2));
                const float3 b = make_float3(__ldg(P.tgt.verts + 3 * (size_t)i1), __ldg(P.tgt.verts + 3 * (size_t)i1 + 1),
                                             __ldg(P.tgt.verts + 3 * (size_t)i1 + 2));
                const float3 c = make_float3(__ldg(P.tgt.verts + 3 * (size_t)i2), __ldg(P.tgt.verts + 3 * (size_t)i2 + 1),
                                             __ldg(P.tgt.verts + 3 * (size_t)i2 + 2));
                if (fminf(a.x, fminf(b.x, c.x)) > p.x || fmaxf(a.x, fmaxf(b.x, c.x)) < p.x ||
                    fminf(a.y, fminf(b.y, c.y)) > p.y || fmaxf(a.y, fmaxf(b.y, c.y)) < p.y ||
                    fmaxf(a.z, fmaxf(b.z, c.z)) < p.z)
                    return;
                ++n_tests;
                if (zray_cross(p, a, b, c, pc)) {
                    crossings ^= 1u;
                    if constexpr (TRACK) ++ncross;
                }
            };
            if (P.tgt.tri_chunk_box) {
                // only the 32-triangle chunks whose box the ray's column meets
                const int64_t end = (int64_t)r.x + r.y;
                const int64_t c_first = (int64_t)r.x / 32, c_last = (end - 1) / 32;
                for (int64_t c0 = c_first; c0 <= c_last; c0 += 32) {
                    const int64_t c = c0 + lane;
                    bool hit = false;
                    if (c <= c_last) {
                        const float* bb = P.tgt.tri_chunk_box + 6 * c;
                        hit = __ldg(bb) <= p.x && p.x <= __ldg(bb + 3) && __ldg(bb + 1) <= p.y &&
                              p.y <= __ldg(bb + 4) && __ldg(bb + 5) >= p.z;
                    }
                    unsigned m = __ballot_sync(0xFFFFFFFFu, hit);
                    while (m) {
                        const int bit = __ffs(m) - 1;
                        m &= m - 1;
                        const int64_t tri = (c0 + bit) * 32 + lane;
                        if (tri >= r.x && tri < end) test(tri);
                    }
                }
            } else {
                for (int k = lane; k < r.y; k += 32) test((int64_t)r.x + k);
            }
            const unsigned odd = __popc(__ballot_sync(0xFFFFFFFFu, crossings != 0)) & 1u;
            if constexpr (TRACK) {
                const uint32_t hits = __reduce_add_sync(0xFFFFFFFFu, ncross);
                if (hits && lane == 0) {
                    ++n_crossed;
                    if (odd) {
                        if (n_odd < (uint32_t)P.track_k) {
                            const int64_t at = s * (int64_t)P.track_k + n_odd;
                            P.track_ids[at] = t;
                            P.track_hits[at] = hits;
                        }
                        ++n_odd;
                    }
                }
            } else if (odd && lane == 0) {
                const uint64_t key = P.swap ? pack_key(t, (int32_t)s) : pack_key((int32_t)s, t);
                uint32_t probes = 0;
                const int64_t slot = hash_insert(P.table, P.mask, key, P.err, probes);
                if (slot >= 0) P.parity[slot] = 1u;  // one warp owns the keys of its source object
            }
        };
        auto finish = [&]() {
            if constexpr (TRACK) {
                if (lane == 0) {
                    P.track_crossed[s] = n_crossed;
                    P.track_overflow[s] = n_odd > (uint32_t)P.track_k ? n_odd - (uint32_t)P.track_k : 0u;
                }
            }
        };
        auto leaf = [&](int first, int count) {
            for (int k = 0; k < count; ++k) {
                const float4 a4 = __ldg(P.objs.soup + 3 * (int64_t)(first + k));
                const float4 b4 = __ldg(P.objs.soup + 3 * (int64_t)(first + k) + 1);
                if (a4.x <= p.x && p.x <= b4.x && a4.y <= p.y && p.y <= b4.y && b4.z >= p.z)
                    candidate(__float_as_int(a4.w));
            }
        };
        if (P.grid.nx > 0) {
            const float* gb = P.grid.bounds;
            int cx, cx1, cy, cy1;
            grid_cell_range(gb, P.grid.nx, P.grid.ny, p.x, p.x, 0, cx, cx1);
            grid_cell_range(gb, P.grid.nx, P.grid.ny, p.y, p.y, 1, cy, cy1);
            const int c = cy * P.grid.nx + cx;
            const int32_t e0 = __ldg(P.grid.offsets + c), e1 = __ldg(P.grid.offsets + c + 1);
            const int32_t part = P.src.obj_part ? __ldg(P.src.obj_part + s) : 0;
            for (int32_t e = e0; e < e1; ++e) {
                const int32_t t = __ldg(P.grid.entries + e);
                if (P.tgt.obj_part && __ldg(P.tgt.obj_part + t) != part) continue;
                const float* ob = P.tgt.obj_box + 6 * (int64_t)t;
                if (__ldg(ob) <= p.x && p.x <= __ldg(ob + 3) && __ldg(ob + 1) <= p.y && p.y <= __ldg(ob + 4) &&
                    __ldg(ob + 5) >= p.z)
                    candidate(t);
            }
            finish();
            continue;
        }
        int first, count;
        int node = traversal_start(P.src, P.objs, (int32_t)s, first, count);
        if (node < 0) {
            leaf(first, count);
            finish();
            continue;
        }
        int stack[kStackSize];
        int sp = 0;
        for (;;) {
            ++n_nodes;
            const Node* nd = P.objs.nodes + node;
            const float4 bx = __ldg(&nd->bx), by = __ldg(&nd->by), bz = __ldg(&nd->bz);
            const int4 ch = __ldg(&nd->ch);
            bool h0 = bx.x <= p.x && p.x <= bx.y && by.x <= p.y && p.y <= by.y && bz.y >= p.z;
            bool h1 = bx.z <= p.x && p.x <= bx.w && by.z <= p.y && p.y <= by.w && bz.w >= p.z;
            if (h0 && ch.x < 0) {
                leaf(~ch.x, ch.z & 0xFF);
                h0 = false;
            }
            if (h1 && ch.y < 0) {
                leaf(~ch.y, (ch.z >> 8) & 0xFF);
                h1 = false;
            }
            if (h0 && h1) {
                if (sp >= kStackSize) {
                    if (lane == 0) atomicOr(P.err, ERR_STACK_OVERFLOW);
                    break;
                }
                stack[sp++] = ch.y;
                node = ch.x;
            } else if (h0) {
                node = ch.x;
            } else if (h1) {
                node = ch.y;
            } else {
                if (sp == 0) break;
                node = stack[--sp];
            }
        }
        finish();
    }
    // per-lane test and ambiguity counts; rays and node visits once per warp
    flush_counter(&P.ctr->tri_tests, n_tests);
    flush_counter(&P.ctr->fp32_ambiguous, pc.fp32_ambiguous);
    flush_counter(&P.ctr->fp64_ambiguous, pc.fp64_ambiguous);
    flush_counter(&P.ctr->parity_rays, lane == 0 ? n_rays : 0u);
    flush_counter(&P.ctr->node_visits, lane == 0 ? n_nodes : 0u);
}

// Column grid of a dataset's object boxes in `mem` (grid_bytes(n) bytes).
size_t column_grid_bytes(int32_t n) {
    const int side = std::max(1, (int)std::ceil(std::sqrt((double)std::max(n, 1))));
    return 16 + 4 * ((size_t)side * side + 1) * 3 + 256;
}

// Column grid, first phase: bounds, per-cell counts and offsets in `mem`;
// *n_entries receives the number of (cell, object) entries.
int column_grid_count(pierce_ctx* ctx, const DevDataset& tgt, void* mem, const int32_t** d_total) {
    const int32_t n = tgt.num_objects;
    const int side = std::max(1, (int)std::ceil(std::sqrt((double)std::max(n, 1))));
    const int cells = side * side;
    char* q = static_cast<char*>(mem);
    uint32_t* ob = reinterpret_cast<uint32_t*>(q);
    float* b = reinterpret_cast<float*>(q);  // decoded in place
    int32_t* counts = reinterpret_cast<int32_t*>(q + 16);
    int32_t* offsets = counts + cells + 1;
    int32_t* cursor = offsets + cells + 1;
    cudaStream_t st = ctx->stream;
    k_fill_u32_j<<<1, 32, 0, st>>>(ob, 0xFFFFFFFFu, 2);
    k_fill_u32_j<<<1, 32, 0, st>>>(ob + 2, 0u, 2);
    cudaMemsetAsync(counts, 0, 4 * ((size_t)cells + 1), st);
    cudaMemsetAsync(cursor, 0, 4 * ((size_t)cells + 1), st);
    if (n > 0) k_grid_bounds<<<grid_cap(ctx, n, 256), 256, 0, st>>>(tgt.obj_box, n, ob);
    k_grid_decode<<<1, 32, 0, st>>>(ob, b);
    if (n > 0)
        k_grid_fill<0><<<grid_cap(ctx, n, 256), 256, 0, st>>>(tgt.obj_box, n, b, side, side, counts, nullptr, nullptr,
                                                               nullptr);
    ctx->launches += 5;
    if (int s = exclusive_scan_i32(ctx, counts, offsets, cells + 1)) return s;
    *d_total = offsets + cells;  // the number of entries, read by the caller
    return PIERCE_OK;
}

// Second phase: the object ids of every cell into `entries` (n_entries).
int column_grid_fill(pierce_ctx* ctx, const DevDataset& tgt, void* mem, int32_t* entries, ColumnGrid* g) {
    const int32_t n = tgt.num_objects;
    const int side = std::max(1, (int)std::ceil(std::sqrt((double)std::max(n, 1))));
    const int cells = side * side;
    char* q = static_cast<char*>(mem);
    float* b = reinterpret_cast<float*>(q);
    int32_t* counts = reinterpret_cast<int32_t*>(q + 16);
    int32_t* offsets = counts + cells + 1;
    int32_t* cursor = offsets + cells + 1;
    if (n > 0) {
        k_grid_fill<1><<<grid_cap(ctx, n, 256), 256, 0, ctx->stream>>>(tgt.obj_box, n, b, side, side, nullptr,
                                                                       offsets, cursor, entries);
        ctx->launches += 1;
    }
    g->nx = side;
    g->ny = side;
    g->bounds = b;
    g->offsets = offsets;
    g->entries = entries;
    return check_cuda(cudaGetLastError(), "column grid");
}

int launch_parity_objects(pierce_ctx* ctx, const DevDataset& src, const DevDataset& objs, const DevDataset& tgt,
                          const ColumnGrid* grid, int swap, uint64_t* table, uint32_t* parity, uint64_t slots,
                          int64_t src_lo, int64_t src_hi) {
    if (src_hi < 0) src_hi = src.num_objects;
    src_lo = std::max<int64_t>(src_lo, 0);
    src_hi = std::min<int64_t>(src_hi, src.num_objects);
    if (src_hi <= src_lo || !tgt.obj_range) return PIERCE_OK;
    ParityObjParams P;
    P.src = src;
    P.src_lo = src_lo;
    P.src_hi = src_hi;
    P.grid = grid ? *grid : ColumnGrid{};
    P.objs = objs;
    P.tgt = tgt;
    P.swap = swap;
    P.table = table;
    P.parity = parity;
    P.mask = slots - 1;
    P.err = ctx->d_err;
    P.ctr = ctx->d_counters;
    P.track_k = 0;
    P.track_ids = nullptr;
    P.track_hits = nullptr;
    P.track_crossed = nullptr;
    P.track_overflow = nullptr;
    const int64_t warps = src_hi - src_lo;
    const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((warps + 3) / 4,
                                                                             (int64_t)ctx->sm_count * 32));
    k_parity_objects<false><<<blocks, 128, 0, ctx->stream>>>(P);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "parity (object pairs) kernel");
}

// Parity-ray diagnostics of src's objects against tgt over tgt's column
// grid: ids[src.num_objects * k] (preset to -1 by the caller), hits (same
// shape), crossed and overflow (src.num_objects each; entries of objects
// without triangles are left as they are).
int launch_parity_tracking(pierce_ctx* ctx, const DevDataset& src, const DevDataset& tgt, const ColumnGrid& grid,
                           int32_t k, int32_t* ids, uint32_t* hits, uint32_t* crossed, uint32_t* overflow) {
    if (src.num_objects <= 0 || !tgt.obj_range || grid.nx <= 0) return PIERCE_OK;
    ParityObjParams P;
    P.src = src;
    P.src_lo = 0;
    P.src_hi = src.num_objects;
    P.grid = grid;
    P.objs = DevDataset{};
    P.tgt = tgt;
    P.swap = 0;
    P.table = nullptr;
    P.parity = nullptr;
    P.mask = 0;
    P.err = ctx->d_err;
    P.ctr = ctx->d_counters;
    P.track_k = k;
    P.track_ids = ids;
    P.track_hits = hits;
    P.track_crossed = crossed;
    P.track_overflow = overflow;
    const int64_t warps = src.num_objects;
    const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((warps + 3) / 4,
                                                                             (int64_t)ctx->sm_count * 32));
    k_parity_objects<true><<<blocks, 128, 0, ctx->stream>>>(P);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "parity tracking kernel");
}

int compact_table(pierce_ctx* ctx, const uint64_t* table, uint64_t slots, uint64_t* out, uint64_t cap,
                  unsigned long long* d_count) {
    k_compact<<<grid_cap(ctx, (int64_t)slots, 256), 256, 0, ctx->stream>>>(table, slots, out, d_count, cap);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "compact kernel");
}

int keys_to_pairs(pierce_ctx* ctx, uint64_t* keys, int64_t n) {
    if (n <= 0) return PIERCE_OK;
    k_keys_to_pairs<<<grid_cap(ctx, n, 256), 256, 0, ctx->stream>>>(keys, n);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "keys_to_pairs");
}

int pairs_to_keys(pierce_ctx* ctx, const uint64_t* pairs, uint64_t* keys, int64_t n) {
    if (n <= 0) return PIERCE_OK;
    k_pairs_to_keys<<<grid_cap(ctx, n, 256), 256, 0, ctx->stream>>>(pairs, keys, n);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "pairs_to_keys");
}

int parity_emit(pierce_ctx* ctx, const uint64_t* ptable, const uint32_t* parity, uint64_t pslots, int mode,
                const uint64_t* lookup_table, uint64_t lookup_slots, const uint64_t* lookup_sorted, int64_t lookup_n,
                uint64_t* out_table, uint64_t out_slots, uint64_t* out_keys, unsigned long long* out_count,
                uint64_t out_cap) {
    k_parity_emit<<<grid_cap(ctx, (int64_t)pslots, 256), 256, 0, ctx->stream>>>(
        ptable, parity, pslots, mode, lookup_table, lookup_slots ? lookup_slots - 1 : 0, lookup_sorted, lookup_n,
        out_table, out_slots ? out_slots - 1 : 0, out_keys, out_count, out_cap, ctx->d_err);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "parity emit");
}

int launch_containment_candidates(pierce_ctx* ctx, const uint64_t* ptable, const uint32_t* parity, uint64_t pslots,
                                  uint8_t* act_a, int64_t na, uint8_t* act_b, int64_t nb) {
    k_mark_candidates<<<grid_cap(ctx, (int64_t)pslots, 256), 256, 0, ctx->stream>>>(ptable, parity, pslots, act_a,
                                                                                   act_b);
    k_keep_candidates<<<grid_cap(ctx, na, 256), 256, 0, ctx->stream>>>(act_a, na);
    k_keep_candidates<<<grid_cap(ctx, nb, 256), 256, 0, ctx->stream>>>(act_b, nb);
    ctx->launches += 3;
    return check_cuda(cudaGetLastError(), "containment candidates");
}

int launch_containment_pairs(pierce_ctx* ctx, const uint64_t* ptable, const uint32_t* parity, uint64_t pslots,
                             const DevDataset& a, const DevDataset& b, uint64_t* out, unsigned long long* count,
                             uint64_t cap, unsigned long long* fallback) {
    if (!a.obj_range || !b.obj_range)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "containment by pairs: objects must be stored contiguously");
    PairParams P;
    P.ptable = ptable;
    P.parity = parity;
    P.pslots = pslots;
    P.a = a;
    P.b = b;
    P.out = out;
    P.count = count;
    P.cap = cap;
    P.fallback = fallback;
    P.ctr = ctx->d_counters;
    const int64_t blocks = std::min<int64_t>(((int64_t)pslots + kPairThreads - 1) / kPairThreads, (int64_t)ctx->sm_count * 8);
    k_containment_pairs<<<(unsigned)std::max<int64_t>(blocks, 1), kPairThreads, 0, ctx->stream>>>(P);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "containment by pairs");
}

// Grid selectivity estimate per matched cell (estimateSelectivityKernel,
// pierce/query/src/cuda/estimated_overlap.cu:8-41): TouchA * TouchB *
// min(1, (sizeA + sizeB + eps)^3 / Vcell * sqrt(ratioA * ratioB)^gamma),
// summed in double.
struct GridCellRec {
    int32_t ix, iy, iz;
    uint32_t center, touch;
    float size, ratio;
};

__global__ void k_estimate(const GridCellRec* __restrict__ a, const GridCellRec* __restrict__ b, int n,
                           float cell_volume, float eps, float gamma, double* total) {
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const GridCellRec A = a[i], B = b[i];
        if (A.touch == 0 || B.touch == 0) continue;
        const float comb = A.size + B.size + eps;
        float prob = comb * comb * comb / cell_volume;
        prob *= powf(sqrtf(A.ratio * B.ratio), gamma);
        prob = fminf(prob, 1.0f);
        acc += (double)((float)A.touch * (float)B.touch * prob);
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xFFFFFFFFu, acc, off);
    if ((threadIdx.x & 31) == 0 && acc != 0.0) atomicAdd(total, acc);
}

int estimate_cells(pierce_ctx* ctx, const void* a, const void* b, int n, float cell_volume, float eps, float gamma,
                   double* total) {
    void* p = nullptr;
    const size_t bytes = sizeof(GridCellRec) * (size_t)n;
    if (int s = scratch(ctx, 7, 2 * bytes + 64, &p)) return s;
    GridCellRec* da = static_cast<GridCellRec*>(p);
    GridCellRec* db = da + n;
    double* dt = reinterpret_cast<double*>(db + n);
    cudaMemcpyAsync(da, a, bytes, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(db, b, bytes, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemsetAsync(dt, 0, sizeof(double), ctx->stream);
    if (cell_volume < 1e-9f) cell_volume = 1e-9f;
    k_estimate<<<grid_cap(ctx, n, 256), 256, 0, ctx->stream>>>(da, db, n, cell_volume, eps, gamma, dt);
    ctx->launches += 1;
    cudaMemcpyAsync(ctx->h_small, dt, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (int s = check_cuda(cudaStreamSynchronize(ctx->stream), "estimate")) return s;
    std::memcpy(total, ctx->h_small, sizeof(double));
    return PIERCE_OK;
}

uint64_t table_slots_for(uint64_t expected, double load_factor) {
    if (load_factor <= 0.0 || load_factor > 1.0) load_factor = 0.5;
    double want = (double)std::max<uint64_t>(expected, 1) / load_factor;
    uint64_t s = next_pow2((uint64_t)std::ceil(want));
    if (s < 1024) s = 1024;
    const uint64_t cap = 1ull << 34;
    if (s > cap) s = cap;
    return s;
}

}  // namespace pgpu
