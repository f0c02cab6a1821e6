// Linear BVH construction over a dataset's triangles (replaces the OptiX
// GAS build of pierce/query/src/optix/OptixAccelerationStructure.cpp:22-68).
//
// Steps, all on the context stream:
//   1. centroids + centroid bounds (block reduction, ordered-integer atomics);
//   2. 30-bit Morton codes of the centroids in the centroid bounds;
//   3. radix sort of (code, triangle) pairs (CUB, sortscan.cu);
//   4. triangle soup in sorted order: 3 float4 per triangle, object id and
//      original index carried in the w lanes;
//   5. hierarchy: Karras 2012 ("Maximizing Parallelism in the Construction
//      of BVHs, Octrees, and k-d Trees"), restated; equal codes are split by
//      index so every node has a unique split and the depth is bounded by
//      30 + 32 levels;
//   6. bottom-up refit: each leaf walks to the root, the second thread to
//      reach a node (atomic arrival counter) merges the two child boxes.
//      Child boxes are stored in the parent (Node::bx/by/bz), which is the
//      layout the traversal reads;
//   7. leaf collapse (in the hierarchy step): children covering <=
//      leaf_size triangles become leaves over their contiguous soup range.
// All box arithmetic is min/max of input floats, so boxes are exact.
#include <cuda/atomic>
#include <cuda_runtime.h>

#include <cstdio>

#include "common.cuh"

namespace pgpu {

__device__ __forceinline__ uint32_t f2o(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__device__ __forceinline__ float3 load_vertex(const float* v, uint32_t i) {
    return make_float3(__ldg(v + 3 * (size_t)i), __ldg(v + 3 * (size_t)i + 1), __ldg(v + 3 * (size_t)i + 2));
}

__global__ void k_fill_u32(uint32_t* p, uint32_t value, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = value;
}

// 1. centroids and their bounds (bounds[0..2] ordered min, [3..5] ordered max)
__global__ void k_centroids(const float* __restrict__ verts, const uint32_t* __restrict__ idx,
                            const uint32_t* __restrict__ list, int64_t nt, float4* __restrict__ cen,
                            uint32_t* __restrict__ bounds) {
    float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nt; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = list ? (int64_t)list[i] : i;
        const float3 a = load_vertex(verts, __ldg(idx + 3 * t));
        const float3 b = load_vertex(verts, __ldg(idx + 3 * t + 1));
        const float3 c = load_vertex(verts, __ldg(idx + 3 * t + 2));
        const float3 m = make_float3((a.x + b.x + c.x) * (1.0f / 3.0f), (a.y + b.y + c.y) * (1.0f / 3.0f),
                                     (a.z + b.z + c.z) * (1.0f / 3.0f));
        cen[i] = make_float4(m.x, m.y, m.z, 0.0f);
        mn[0] = fminf(mn[0], m.x); mn[1] = fminf(mn[1], m.y); mn[2] = fminf(mn[2], m.z);
        mx[0] = fmaxf(mx[0], m.x); mx[1] = fmaxf(mx[1], m.y); mx[2] = fmaxf(mx[2], m.z);
    }
    // warp, then block reduction: one set of six atomics per block
    __shared__ float red[2][3][32];
    for (int k = 0; k < 3; ++k) {
        for (int off = 16; off > 0; off >>= 1) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], off));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], off));
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0)
        for (int k = 0; k < 3; ++k) {
            red[0][k][wid] = mn[k];
            red[1][k][wid] = mx[k];
        }
    __syncthreads();
    if (wid == 0) {
        for (int k = 0; k < 3; ++k) {
            float a = lane < nw ? red[0][k][lane] : 3.4e38f, b = lane < nw ? red[1][k][lane] : -3.4e38f;
            for (int off = 16; off > 0; off >>= 1) {
                a = fminf(a, __shfl_xor_sync(0xFFFFFFFFu, a, off));
                b = fmaxf(b, __shfl_xor_sync(0xFFFFFFFFu, b, off));
            }
            if (lane == 0) {
                atomicMin(bounds + k, f2o(a));
                atomicMax(bounds + 3 + k, f2o(b));
            }
        }
    }
}

__device__ __forceinline__ uint32_t expand_bits10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// 2. Morton codes
__global__ void k_morton(const float4* __restrict__ cen, int64_t nt, const uint32_t* __restrict__ bounds,
                         uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const float lo[3] = {o2f(bounds[0]), o2f(bounds[1]), o2f(bounds[2])};
    const float hi[3] = {o2f(bounds[3]), o2f(bounds[4]), o2f(bounds[5])};
    float inv[3];
    for (int k = 0; k < 3; ++k) inv[k] = hi[k] > lo[k] ? 1.0f / (hi[k] - lo[k]) : 0.0f;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
        const float4 c = cen[t];
        const float cc[3] = {c.x, c.y, c.z};
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) {
            float u = (cc[k] - lo[k]) * inv[k];
            u = fminf(fmaxf(u, 0.0f), 1.0f);
            q[k] = min((uint32_t)(u * 1024.0f), 1023u);
        }
        keys[t] = (expand_bits10(q[0]) << 2) | (expand_bits10(q[1]) << 1) | expand_bits10(q[2]);
        vals[t] = (uint32_t)t;
    }
}

// 1'/2'. partitioned hierarchy: centroid bounds per partition (warps whose
// lanes share a partition reduce in registers first), then 64-bit keys
// (partition << 30 | Morton code in the partition's bounds).
__global__ void k_centroids_parts(const float* __restrict__ verts, const uint32_t* __restrict__ idx,
                                  const uint32_t* __restrict__ list, const int32_t* __restrict__ t2o,
                                  const int32_t* __restrict__ obj_part, int64_t nt, float4* __restrict__ cen,
                                  uint32_t* __restrict__ bounds) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < nt; base += stride) {
        const int64_t i = base + threadIdx.x;
        int32_t part = -1;
        float m[3] = {0.0f, 0.0f, 0.0f};
        if (i < nt) {
            const int64_t t = list ? (int64_t)list[i] : i;
            const float3 a = load_vertex(verts, __ldg(idx + 3 * t));
            const float3 b = load_vertex(verts, __ldg(idx + 3 * t + 1));
            const float3 c = load_vertex(verts, __ldg(idx + 3 * t + 2));
            m[0] = (a.x + b.x + c.x) * (1.0f / 3.0f);
            m[1] = (a.y + b.y + c.y) * (1.0f / 3.0f);
            m[2] = (a.z + b.z + c.z) * (1.0f / 3.0f);
            part = __ldg(obj_part + __ldg(t2o + t));
            cen[i] = make_float4(m[0], m[1], m[2], __int_as_float(part));
        }
        const int32_t p0 = __shfl_sync(0xFFFFFFFFu, part, 0);
        if (__all_sync(0xFFFFFFFFu, part == p0 || part < 0) && p0 >= 0) {
            float mn[3] = {m[0], m[1], m[2]}, mx[3] = {m[0], m[1], m[2]};
            if (part < 0)
                for (int k = 0; k < 3; ++k) {
                    mn[k] = 3.4e38f;
                    mx[k] = -3.4e38f;
                }
            for (int k = 0; k < 3; ++k)
                for (int off = 16; off > 0; off >>= 1) {
                    mn[k] = fminf(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], off));
                    mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], off));
                }
            if ((threadIdx.x & 31) == 0)
                for (int k = 0; k < 3; ++k) {
                    atomicMin(bounds + 6 * (int64_t)p0 + k, f2o(mn[k]));
                    atomicMax(bounds + 6 * (int64_t)p0 + 3 + k, f2o(mx[k]));
                }
        } else if (part >= 0) {
            for (int k = 0; k < 3; ++k) {
                atomicMin(bounds + 6 * (int64_t)part + k, f2o(m[k]));
                atomicMax(bounds + 6 * (int64_t)part + 3 + k, f2o(m[k]));
            }
        }
    }
}

__global__ void k_morton_parts(const float4* __restrict__ cen, int64_t nt, const uint32_t* __restrict__ bounds,
                               uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
        const float4 c = cen[t];
        const int32_t part = __float_as_int(c.w);
        const uint32_t* b = bounds + 6 * (int64_t)part;
        const float cc[3] = {c.x, c.y, c.z};
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) {
            const float lo = o2f(b[k]), hi = o2f(b[3 + k]);
            const float inv = hi > lo ? 1.0f / (hi - lo) : 0.0f;
            float u = (cc[k] - lo) * inv;
            u = fminf(fmaxf(u, 0.0f), 1.0f);
            q[k] = min((uint32_t)(u * 1024.0f), 1023u);
        }
        const uint32_t code = (expand_bits10(q[0]) << 2) | (expand_bits10(q[1]) << 1) | expand_bits10(q[2]);
        keys[t] = ((uint64_t)(uint32_t)part << 30) | code;
        vals[t] = (uint32_t)t;
    }
}

__global__ void k_fill_roots(int2* roots, int32_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        roots[i] = make_int2(-1, 0);
}

// a one-triangle partitioned hierarchy: its partition's root is that leaf
__global__ void k_single_part_root(const uint64_t* keys, int2* roots) {
    roots[keys[0] >> 30] = make_int2(~0, 1);
}

// 4. triangle soup in sorted order
__global__ void k_soup(const float* __restrict__ verts, const uint32_t* __restrict__ idx,
                       const int32_t* __restrict__ t2o, const uint32_t* __restrict__ list,
                       const uint32_t* __restrict__ order, int64_t nt, float4* __restrict__ soup) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nt; j += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t t = list ? list[order[j]] : order[j];
        const float3 a = load_vertex(verts, __ldg(idx + 3 * (size_t)t));
        const float3 b = load_vertex(verts, __ldg(idx + 3 * (size_t)t + 1));
        const float3 c = load_vertex(verts, __ldg(idx + 3 * (size_t)t + 2));
        soup[3 * j + 0] = make_float4(a.x, a.y, a.z, __int_as_float(__ldg(t2o + t)));
        soup[3 * j + 1] = make_float4(b.x, b.y, b.z, __int_as_float((int)t));
        soup[3 * j + 2] = make_float4(c.x, c.y, c.z, 0.0f);
    }
}

// longest common prefix of sorted keys i and j (index tie-break), -1 outside
__device__ __forceinline__ int lcp(const uint32_t* keys, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t ki = keys[i], kj = keys[j];
    if (ki == kj) return 32 + __clzll((unsigned long long)(i ^ j)) - 32;  // 32 + clz over 32-bit index
    return __clz(ki ^ kj);
}
__device__ __forceinline__ int lcp(const uint64_t* keys, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    const uint64_t ki = keys[i], kj = keys[j];
    if (ki == kj) return 64 + __clzll((unsigned long long)(i ^ j));
    return __clzll(ki ^ kj);
}

// partition of sorted key k (32-bit keys carry none)
__device__ __forceinline__ uint32_t key_part(const uint32_t*, int64_t) { return 0u; }
__device__ __forceinline__ uint32_t key_part(const uint64_t* keys, int64_t k) { return (uint32_t)(keys[k] >> 30); }

// 5. Karras hierarchy with leaf collapse.  Internal node i covers the
// sorted range [first, last]; a child whose range holds <= leaf_size
// triangles becomes a leaf over that range, and nodes inside such a range
// are never created.  Links for the refit are written here:
//   * node.ch.w of an internal child = parent << 2 | side << 1 (bit 0 is the
//     arrival toggle, initially 0; the root's parent is kRootParent);
//   * leaf_rec[first] of a leaf child = parent << 9 | side << 8 | count.
// Every word is written by exactly one thread (ch.x/y/z by the node's own
// thread, ch.w by its parent's thread), so no two threads write one word.
constexpr uint32_t kRootParent = 0x3FFFFFFFu;

//
// Partitioned keys: a range is collapsed into a leaf only when it lies in
// one partition, and every range that is exactly one whole partition
// records itself in part_roots (an internal node, or a leaf child).  The
// keys of one partition share their partition bits, so they form one
// subtree of the radix tree.
template <typename K>
__global__ void k_karras(const K* __restrict__ keys, int64_t n, int leaf_size, Node* __restrict__ nodes,
                         unsigned long long* __restrict__ leaf_rec, int2* __restrict__ part_roots) {
    auto whole_part = [&](int64_t f, int64_t l) {
        const uint32_t p = key_part(keys, f);
        return key_part(keys, l) == p && (f == 0 || key_part(keys, f - 1) != p) &&
               (l == n - 1 || key_part(keys, l + 1) != p);
    };
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n - 1; i += (int64_t)gridDim.x * blockDim.x) {
        const int d = (lcp(keys, n, i, i + 1) - lcp(keys, n, i, i - 1)) >= 0 ? 1 : -1;
        const int dmin = lcp(keys, n, i, i - d);
        int64_t lmax = 2;
        while (lcp(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
        int64_t l = 0;
        for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
            if (lcp(keys, n, i, i + (l + t) * d) > dmin) l += t;
        const int64_t j = i + l * d;
        const int64_t first = i < j ? i : j, last = i < j ? j : i;
        if (i != 0 && last - first + 1 <= leaf_size && key_part(keys, first) == key_part(keys, last))
            continue;  // inside a collapsed leaf
        if (part_roots && whole_part(first, last)) part_roots[key_part(keys, first)] = make_int2((int)i, 0);
        const int dnode = lcp(keys, n, i, j);
        int64_t s = 0, t = l;
        do {
            t = (t + 1) >> 1;
            if (lcp(keys, n, i, i + (s + t) * d) > dnode) s += t;
        } while (t > 1);
        const int64_t gamma = i + s * d + (d < 0 ? -1 : 0);
        int child[2];
        int count[2] = {0, 0};
        const int64_t cfirst[2] = {first, gamma + 1}, clast[2] = {gamma, last};
        const int64_t cidx[2] = {gamma, gamma + 1};
        for (int side = 0; side < 2; ++side) {
            const int64_t size = clast[side] - cfirst[side] + 1;
            if (size <= leaf_size && key_part(keys, cfirst[side]) == key_part(keys, clast[side])) {
                child[side] = ~(int)cfirst[side];
                count[side] = (int)size;
                leaf_rec[cfirst[side]] = ((unsigned long long)i << 9) | ((unsigned long long)side << 8) |
                                         (unsigned long long)size;
                if (part_roots && whole_part(cfirst[side], clast[side]))
                    part_roots[key_part(keys, cfirst[side])] = make_int2(~(int)cfirst[side], (int)size);
            } else {
                child[side] = (int)cidx[side];
                nodes[cidx[side]].ch.w = (int)(((uint32_t)i << 2) | ((uint32_t)side << 1));
            }
        }
        Node* nd = nodes + i;
        nd->ch.x = child[0];
        nd->ch.y = child[1];
        nd->ch.z = count[0] | (count[1] << 8);
        if (i == 0) nd->ch.w = (int)(kRootParent << 2);
    }
}

__device__ __forceinline__ void store_child_box(Node* nd, int slot, const float lo[3], const float hi[3]) {
    float* bx = reinterpret_cast<float*>(&nd->bx);
    float* by = reinterpret_cast<float*>(&nd->by);
    float* bz = reinterpret_cast<float*>(&nd->bz);
    __stcg(bx + 2 * slot, lo[0]);
    __stcg(bx + 2 * slot + 1, hi[0]);
    __stcg(by + 2 * slot, lo[1]);
    __stcg(by + 2 * slot + 1, hi[1]);
    __stcg(bz + 2 * slot, lo[2]);
    __stcg(bz + 2 * slot + 1, hi[2]);
}
__device__ __forceinline__ void load_child_box(Node* nd, int slot, float lo[3], float hi[3]) {
    const float* bx = reinterpret_cast<const float*>(&nd->bx);
    const float* by = reinterpret_cast<const float*>(&nd->by);
    const float* bz = reinterpret_cast<const float*>(&nd->bz);
    lo[0] = __ldcg(bx + 2 * slot);
    hi[0] = __ldcg(bx + 2 * slot + 1);
    lo[1] = __ldcg(by + 2 * slot);
    hi[1] = __ldcg(by + 2 * slot + 1);
    lo[2] = __ldcg(bz + 2 * slot);
    hi[2] = __ldcg(bz + 2 * slot + 1);
}

// 6. refit: the first levels in waves, the rest in chains.  The leaf wave
// computes each leaf's box, stores it in its parent's child slot and flips
// the parent's arrival toggle; the second arrival appends the parent to a
// list.  Each following wave takes the list of nodes whose two child slots
// are complete, merges them, stores the result in the grandparent and
// appends it the same way.  A node is only read in the wave after the one
// that completed it, so kernel boundaries order the box stores and loads and
// these toggles need no memory fence; every wave runs full warps.  After a
// few waves the remaining nodes (a small fraction near the top) finish in
// one chain launch (k_refit_chain).
__device__ __forceinline__ void block_append(bool has, uint32_t value, uint32_t* out, unsigned long long* count) {
    __shared__ uint32_t warp_tot[32];
    __shared__ unsigned long long base;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nwarps = blockDim.x >> 5;
    const unsigned ballot = __ballot_sync(0xFFFFFFFFu, has);
    if (lane == 0) warp_tot[wid] = __popc(ballot);
    __syncthreads();
    if (wid == 0) {
        uint32_t w = lane < nwarps ? warp_tot[lane] : 0;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, w, off);
            if (lane >= off) w += v;
        }
        if (lane < nwarps) warp_tot[lane] = w;
        if (lane == 31) base = w ? atomicAdd(count, (unsigned long long)w) : 0ull;
    }
    __syncthreads();
    if (has) out[base + (wid ? warp_tot[wid - 1] : 0u) + __popc(ballot & ((1u << lane) - 1u))] = value;
    __syncthreads();
}

__device__ __forceinline__ void write_slot(Node* nd, int slot, const float lo[3], const float hi[3]) {
    float* bx = reinterpret_cast<float*>(&nd->bx);
    float* by = reinterpret_cast<float*>(&nd->by);
    float* bz = reinterpret_cast<float*>(&nd->bz);
    bx[2 * slot] = lo[0];
    bx[2 * slot + 1] = hi[0];
    by[2 * slot] = lo[1];
    by[2 * slot + 1] = hi[1];
    bz[2 * slot] = lo[2];
    bz[2 * slot + 1] = hi[2];
}

// Store a finished box into node `node`'s slot `side`; true when this was the
// second arrival (the node is then complete).
__device__ __forceinline__ bool deliver(Node* nodes, uint32_t node, int side, const float lo[3], const float hi[3]) {
    Node* nd = nodes + node;
    write_slot(nd, side, lo, hi);
    return (atomicXor(reinterpret_cast<unsigned int*>(&nd->ch.w), 1u) & 1u) != 0u;
}

__global__ void __launch_bounds__(256) k_refit_leaves(const float4* __restrict__ soup, int64_t n, Node* nodes,
                                                      const unsigned long long* __restrict__ leaf_rec,
                                                      uint32_t* list_out, unsigned long long* count_out) {
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = base + threadIdx.x;
        bool done = false, bad_leaf = false;
        uint32_t node = 0;
        if (j < n) {
            const unsigned long long rec = leaf_rec[j];
            if (rec != ~0ull) {
                const int count = (int)(rec & 0xFF);
                const int side = (int)((rec >> 8) & 1);
                node = (uint32_t)(rec >> 9);
                float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
                if ((int64_t)node >= n - 1 || j + count > n) bad_leaf = true;
                for (int k = 0; k < count && !bad_leaf; ++k)
                    for (int v = 0; v < 3; ++v) {
                        const float4 p = soup[3 * (j + k) + v];
                        lo[0] = fminf(lo[0], p.x);
                        lo[1] = fminf(lo[1], p.y);
                        lo[2] = fminf(lo[2], p.z);
                        hi[0] = fmaxf(hi[0], p.x);
                        hi[1] = fmaxf(hi[1], p.y);
                        hi[2] = fmaxf(hi[2], p.z);
                    }
                if (!bad_leaf) done = deliver(nodes, node, side, lo, hi);
            }
        }
        block_append(done, node, list_out, count_out);
    }
}

__global__ void __launch_bounds__(256) k_refit_wave(Node* nodes, int64_t num_nodes, const uint32_t* __restrict__ list_in,
                                                    const unsigned long long* __restrict__ count_in, int64_t list_cap,
                                                    uint32_t* list_out, unsigned long long* count_out,
                                                    float* root_box) {
    int64_t n = (int64_t)*count_in;
    if (n > list_cap) n = list_cap;  // never read past the list
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = base + threadIdx.x;
        bool done = false;
        uint32_t parent = 0;
        if (i < n && (int64_t)list_in[i] < num_nodes) {
            const Node* nd = nodes + list_in[i];
            const float4 bx = nd->bx, by = nd->by, bz = nd->bz;
            const uint32_t w = (uint32_t)nd->ch.w;
            const float lo[3] = {fminf(bx.x, bx.z), fminf(by.x, by.z), fminf(bz.x, bz.z)};
            const float hi[3] = {fmaxf(bx.y, bx.w), fmaxf(by.y, by.w), fmaxf(bz.y, bz.w)};
            parent = w >> 2;
            if (parent == kRootParent) {
                for (int k = 0; k < 3; ++k) {
                    root_box[k] = lo[k];
                    root_box[3 + k] = hi[k];
                }
            } else if ((int64_t)parent < num_nodes) {
                done = deliver(nodes, parent, (int)((w >> 1) & 1u), lo, hi);
            }
        }
        block_append(done, parent, list_out, count_out);
    }
}

// Chains from the last wave's list: each listed node (both slots complete)
// merges its slots and delivers the box to its parent with an
// acquire-release flip of the parent's toggle: the release makes the box
// visible before the flip, the acquire lets the second arrival see its
// sibling's box (delivered in this launch or an earlier one).  The first
// arrival stops; the second merges and carries on upward, so every node is
// completed by exactly one thread and no thread waits.  A chain is at most
// the tree height long; the step bound only guards against a corrupt tree.
__global__ void __launch_bounds__(256) k_refit_chain(Node* nodes, int64_t num_nodes,
                                                     const uint32_t* __restrict__ list,
                                                     const unsigned long long* __restrict__ count, int64_t list_cap,
                                                     float* root_box, uint32_t* err) {
    int64_t n = (int64_t)*count;
    if (n > list_cap) n = list_cap;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t node = list[i];
        if ((int64_t)node >= num_nodes) {
            atomicOr(err, ERR_STACK_OVERFLOW);
            continue;
        }
        float lo[3], hi[3], l2[3], h2[3];
        Node* nd = nodes + node;
        load_child_box(nd, 0, lo, hi);
        load_child_box(nd, 1, l2, h2);
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], l2[k]);
            hi[k] = fmaxf(hi[k], h2[k]);
        }
        uint32_t w = (uint32_t)__ldcg(&nd->ch.w);
        for (int step = 0;; ++step) {
            const uint32_t parent = w >> 2;
            if (parent == kRootParent) {
                for (int k = 0; k < 3; ++k) {
                    root_box[k] = lo[k];
                    root_box[3 + k] = hi[k];
                }
                break;
            }
            if ((int64_t)parent >= num_nodes || step >= 256) {
                atomicOr(err, ERR_STACK_OVERFLOW);
                break;
            }
            Node* pn = nodes + parent;
            store_child_box(pn, (int)((w >> 1) & 1u), lo, hi);
            cuda::atomic_ref<unsigned int, cuda::thread_scope_device> toggle(
                *reinterpret_cast<unsigned int*>(&pn->ch.w));
            const unsigned int old = toggle.fetch_xor(1u, cuda::memory_order_acq_rel);
            if ((old & 1u) == 0u) break;  // first arrival: the sibling's chain continues
            load_child_box(pn, 0, lo, hi);
            load_child_box(pn, 1, l2, h2);
            for (int k = 0; k < 3; ++k) {
                lo[k] = fminf(lo[k], l2[k]);
                hi[k] = fmaxf(hi[k], h2[k]);
            }
            w = old;
        }
    }
}

// whole dataset in one leaf (n <= leaf_size): root box over all triangles
__global__ void k_single_box(const float4* __restrict__ soup, int64_t n, float* root_box) {
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int64_t t = 0; t < 3 * n; ++t) {
        const float4 p = soup[t];
        lo[0] = fminf(lo[0], p.x);
        lo[1] = fminf(lo[1], p.y);
        lo[2] = fminf(lo[2], p.z);
        hi[0] = fmaxf(hi[0], p.x);
        hi[1] = fmaxf(hi[1], p.y);
        hi[2] = fmaxf(hi[2], p.z);
    }
    for (int k = 0; k < 3; ++k) {
        root_box[k] = lo[k];
        root_box[3 + k] = hi[k];
    }
}

// ---- per-object data: first vertex, bounding box ------------------------

// Triangle chunk boxes (the box of every 32 consecutive triangles) and, per
// object, its lowest and highest triangle index, triangle count and box, in
// one pass over the triangles.  Each warp reads a contiguous range of chunks
// and carries the running aggregate of the object whose triangles it is
// reading (a chunk whose 32 triangles all belong to one object contributes
// its chunk box); the aggregate goes to memory with atomics only when the
// object changes and at the end of the range, so an object of many
// consecutive triangles costs a few atomics per warp that reads it instead
// of a handful per 32 triangles (thousands of warps adding to one counter
// serialise in L2).  Chunks that mix objects, or hold invalid object ids,
// update per triangle.  chunk_box may be null.
__global__ void __launch_bounds__(256) k_prepare_tris(const float* __restrict__ verts, const uint32_t* __restrict__ idx,
                                                      const int32_t* __restrict__ t2o, int64_t nt, int32_t nobj,
                                                      float* __restrict__ chunk_box, int32_t* first_tri,
                                                      int32_t* last, int32_t* count, uint32_t* obj_box_o) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int64_t chunks = (nt + 31) / 32;
    const int64_t c0 = chunks * w / nwarps, c1 = chunks * (w + 1) / nwarps;
    // the carried aggregate (the same in every lane)
    int32_t cur = -1, cfirst = 0, clast = 0, ccount = 0;
    float cmn[3] = {0, 0, 0}, cmx[3] = {0, 0, 0};
    auto flush = [&]() {
        if (cur >= 0 && lane == 0) {
            atomicMin(first_tri + cur, cfirst);
            atomicMax(last + cur, clast);
            atomicAdd(count + cur, ccount);
            uint32_t* bx = obj_box_o + 6 * (size_t)cur;
            for (int k = 0; k < 3; ++k) {
                atomicMin(bx + k, f2o(cmn[k]));
                atomicMax(bx + 3 + k, f2o(cmx[k]));
            }
        }
        cur = -1;
    };
    for (int64_t c = c0; c < c1; ++c) {
        const int64_t t = c * 32 + lane;
        const bool valid = t < nt;
        int32_t o = valid ? __ldg(t2o + t) : -1;
        if (o >= nobj) o = -1;
        float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
        if (valid) {
            for (int v = 0; v < 3; ++v) {
                const float3 p = load_vertex(verts, __ldg(idx + 3 * t + v));
                mn[0] = fminf(mn[0], p.x); mn[1] = fminf(mn[1], p.y); mn[2] = fminf(mn[2], p.z);
                mx[0] = fmaxf(mx[0], p.x); mx[1] = fmaxf(mx[1], p.y); mx[2] = fmaxf(mx[2], p.z);
            }
        }
        float lo[3] = {mn[0], mn[1], mn[2]}, hi[3] = {mx[0], mx[1], mx[2]};
        for (int k = 0; k < 3; ++k)
            for (int off = 16; off > 0; off >>= 1) {
                lo[k] = fminf(lo[k], __shfl_xor_sync(0xFFFFFFFFu, lo[k], off));
                hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xFFFFFFFFu, hi[k], off));
            }
        if (chunk_box && lane < 6) chunk_box[6 * c + lane] = lane < 3 ? lo[lane] : hi[lane - 3];
        const int32_t o0 = __shfl_sync(0xFFFFFFFFu, o, 0);
        if (__all_sync(0xFFFFFFFFu, o == o0) && o0 >= 0) {
            // every triangle of the chunk belongs to o0: the chunk box is its share
            if (o0 != cur) {
                flush();
                cur = o0;
                cfirst = (int32_t)(c * 32);
                clast = (int32_t)(c * 32 + 31);
                ccount = 0;
                for (int k = 0; k < 3; ++k) {
                    cmn[k] = lo[k];
                    cmx[k] = hi[k];
                }
            }
            cfirst = min(cfirst, (int32_t)(c * 32));
            clast = max(clast, (int32_t)(c * 32 + 31));
            ccount += 32;
            for (int k = 0; k < 3; ++k) {
                cmn[k] = fminf(cmn[k], lo[k]);
                cmx[k] = fmaxf(cmx[k], hi[k]);
            }
        } else if (o >= 0) {
            atomicMin(first_tri + o, (int32_t)t);
            atomicMax(last + o, (int32_t)t);
            atomicAdd(count + o, 1);
            uint32_t* bx = obj_box_o + 6 * (size_t)o;
            for (int k = 0; k < 3; ++k) {
                atomicMin(bx + k, f2o(mn[k]));
                atomicMax(bx + 3 + k, f2o(mx[k]));
            }
        }
    }
    flush();
}

__global__ void k_obj_finish(const int32_t* __restrict__ first_tri, const int32_t* __restrict__ count,
                             const int32_t* __restrict__ last, int32_t nobj, int64_t nv,
                             const float* __restrict__ verts, const uint32_t* __restrict__ idx, float4* first_vertex,
                             uint32_t* obj_box_o, int2* obj_range, int32_t* contiguous) {
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < nobj; o += (int64_t)gridDim.x * blockDim.x) {
        const int32_t t = first_tri[o];
        const int32_t c = count[o];
        obj_range[o] = make_int2(c > 0 ? t : 0, c);
        if (c > 0 && last[o] - t + 1 != c) atomicAnd(contiguous, 0);
        float4 fv = make_float4(0.0f, 0.0f, 0.0f, 1.0f);  // w = 1: object has no triangle
        if (t != 0x7FFFFFFF) {
            const uint32_t vi = idx[3 * (size_t)t];
            if (vi < nv) {
                const float3 v = load_vertex(verts, vi);
                fv = make_float4(v.x, v.y, v.z, 0.0f);
            }
        }
        first_vertex[o] = fv;
        float* out = reinterpret_cast<float*>(obj_box_o + 6 * (size_t)o);
        for (int k = 0; k < 6; ++k) out[k] = o2f(obj_box_o[6 * (size_t)o + k]);
    }
}

// Clears *flag when edge sources ever decrease (edges not grouped by object).
__global__ void k_edges_grouped(const int32_t* __restrict__ src, int64_t ne, int32_t* flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x + 1; i < ne; i += (int64_t)gridDim.x * blockDim.x)
        if (__ldg(src + i) < __ldg(src + i - 1)) atomicAnd(flag, 0);
}

__global__ void k_obj_box_init(uint32_t* box_o, int32_t nobj) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 6 * (int64_t)nobj;
         i += (int64_t)gridDim.x * blockDim.x)
        box_o[i] = (i % 6) < 3 ? f2o(__int_as_float(0x7F800000)) : f2o(__int_as_float((int)0xFF800000u));
}

static inline int grid_for(pierce_ctx* ctx, int64_t n, int block) {
    int64_t blocks = (n + block - 1) / block;
    int64_t cap = (int64_t)ctx->sm_count * 16;
    if (blocks > cap) blocks = cap;
    return (int)(blocks < 1 ? 1 : blocks);
}

// Boxes of every 32 consecutive triangles (EDGES = false) or edges: a warp
// per chunk, one item per lane, reduced with shuffles.
template <bool EDGES>
__global__ void __launch_bounds__(256) k_chunk_boxes(const float* __restrict__ verts, const uint32_t* __restrict__ idx,
                                                     const float4* __restrict__ edges, int64_t n,
                                                     float* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t chunks = (n + 31) / 32;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t c = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < chunks; c += warps) {
        const int64_t i = c * 32 + lane;
        float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
        if (i < n) {
            if (EDGES) {
                const float4 a = __ldg(edges + 2 * i), b = __ldg(edges + 2 * i + 1);
                lo[0] = fminf(a.x, b.x); lo[1] = fminf(a.y, b.y); lo[2] = fminf(a.z, b.z);
                hi[0] = fmaxf(a.x, b.x); hi[1] = fmaxf(a.y, b.y); hi[2] = fmaxf(a.z, b.z);
            } else {
                for (int v = 0; v < 3; ++v) {
                    const float3 p = load_vertex(verts, __ldg(idx + 3 * i + v));
                    lo[0] = fminf(lo[0], p.x); lo[1] = fminf(lo[1], p.y); lo[2] = fminf(lo[2], p.z);
                    hi[0] = fmaxf(hi[0], p.x); hi[1] = fmaxf(hi[1], p.y); hi[2] = fmaxf(hi[2], p.z);
                }
            }
        }
        for (int k = 0; k < 3; ++k)
            for (int off = 16; off > 0; off >>= 1) {
                lo[k] = fminf(lo[k], __shfl_xor_sync(0xFFFFFFFFu, lo[k], off));
                hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xFFFFFFFFu, hi[k], off));
            }
        if (lane < 6) out[6 * c + lane] = lane < 3 ? lo[lane] : hi[lane - 3];
    }
}

int prepare_objects(pierce_ctx* ctx, pierce_dataset* ds, cudaEvent_t edges_ready, const int32_t* grouped_flag) {
    const int32_t nobj = ds->num_objects;
    {
        cudaStream_t st = ctx->stream;
        const int64_t ec = (int64_t)(ds->ne + 31) / 32;
        if (!edges_ready && ec > 0 && ds->d_edge_chunk_box) {
            k_chunk_boxes<true><<<grid_for(ctx, 32 * ec, 256), 256, 0, st>>>(nullptr, nullptr, ds->d_edges,
                                                                             (int64_t)ds->ne, ds->d_edge_chunk_box);
            ctx->launches += 1;
        }
    }
    if (nobj <= 0) {
        // no objects: the triangle chunk boxes alone
        const int64_t tc = (int64_t)(ds->nt + 31) / 32;
        if (tc > 0 && ds->d_tri_chunk_box) {
            k_chunk_boxes<false><<<grid_for(ctx, 32 * tc, 256), 256, 0, ctx->stream>>>(
                ds->d_vertices, ds->d_indices, nullptr, (int64_t)ds->nt, ds->d_tri_chunk_box);
            ctx->launches += 1;
        }
        if (edges_ready) return check_cuda(cudaStreamWaitEvent(ctx->stream, edges_ready, 0), "upload wait");
        return PIERCE_OK;
    }
    void* p = nullptr;
    // first triangle, count, last triangle per object, then the contiguity flag
    if (int s = scratch(ctx, 1, sizeof(int32_t) * (3 * (size_t)nobj + 4), &p)) return s;
    int32_t* first_tri = static_cast<int32_t*>(p);
    int32_t* count = first_tri + nobj;
    int32_t* last = count + nobj;
    int32_t* flag = last + nobj;
    uint32_t* box_o = reinterpret_cast<uint32_t*>(ds->d_obj_box);
    cudaStream_t st = ctx->stream;
    k_fill_u32<<<grid_for(ctx, nobj, 256), 256, 0, st>>>(reinterpret_cast<uint32_t*>(first_tri), 0x7FFFFFFFu, nobj);
    cudaMemsetAsync(count, 0, sizeof(int32_t) * (size_t)nobj, st);
    k_fill_u32<<<grid_for(ctx, nobj, 256), 256, 0, st>>>(reinterpret_cast<uint32_t*>(last), 0xFFFFFFFFu, nobj);
    k_fill_u32<<<1, 32, 0, st>>>(reinterpret_cast<uint32_t*>(flag), 1u, 2);
    if (ds->ne > 1 && !grouped_flag) {
        k_edges_grouped<<<grid_for(ctx, (int64_t)ds->ne, 256), 256, 0, st>>>(ds->d_edge_src, (int64_t)ds->ne, flag + 1);
        ctx->launches += 1;
    }
    k_obj_box_init<<<grid_for(ctx, 6 * (int64_t)nobj, 256), 256, 0, st>>>(box_o, nobj);
    if (ds->nt > 0) {
        // one warp per range of chunks: a multiple of the SMs' warp slots
        const int64_t tc = (int64_t)(ds->nt + 31) / 32;
        const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((tc + 7) / 8, (int64_t)ctx->sm_count * 8));
        k_prepare_tris<<<(unsigned)blocks, 256, 0, st>>>(ds->d_vertices, ds->d_indices, ds->d_tri_to_object,
                                                         (int64_t)ds->nt, nobj, ds->d_tri_chunk_box, first_tri, last,
                                                         count, box_o);
    }
    k_obj_finish<<<grid_for(ctx, nobj, 256), 256, 0, st>>>(first_tri, count, last, nobj, (int64_t)ds->nv,
                                                            ds->d_vertices, ds->d_indices, ds->d_first_vertex, box_o,
                                                            ds->d_obj_range, flag);
    ctx->launches += 5 + (ds->nt > 0 ? 1 : 0);
    if (int s = check_cuda(cudaGetLastError(), "prepare_objects")) return s;
    // the edge side (uploaded on the copy stream) must have arrived
    if (edges_ready)
        if (int s = check_cuda(cudaStreamWaitEvent(st, edges_ready, 0), "upload wait")) return s;
    int64_t contiguous = 0, grouped = 0;
    if (int s = host_value(ctx, flag, 4, &contiguous, "object ranges")) return s;
    if (int s = host_value(ctx, grouped_flag ? grouped_flag : flag + 1, 4, &grouped, "edge order")) return s;
    ds->contiguous = contiguous != 0;
    ds->edges_grouped = grouped != 0;
    return PIERCE_OK;
}

// Triangles -> LBVH.  The n triangles are idx[3t..3t+2] for t = list[i]
// (or t = i without a list); soup and nodes receive the structure; build
// temporaries live in scratch slots 1..4.  Everything is enqueued on the
// context stream; when root_box is non-null the root box is read back
// (synchronously).
int build_lbvh(pierce_ctx* ctx, const float* verts, const uint32_t* idx, const int32_t* t2o, const uint32_t* list,
               int64_t n, int leaf_size, float4* soup, Node* nodes, BvhShape* shape, float* root_box,
               const int32_t* obj_part, int32_t num_parts, int2* part_roots) {
    cudaStream_t st = ctx->stream;
    if (leaf_size < 1) leaf_size = 1;
    if (leaf_size > 16) leaf_size = 16;
    shape->leaf_size = leaf_size;
    if (n >= (int64_t(1) << 30))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "bvh build: at most 2^30 - 1 triangles per hierarchy");
    const bool parts = obj_part && num_parts > 0 && part_roots;
    if (parts) {
        k_fill_roots<<<grid_for(ctx, num_parts, 256), 256, 0, st>>>(part_roots, num_parts);
        ctx->launches += 1;
    }
    if (n == 0) {
        shape->root_is_leaf = 1;
        shape->root_leaf_count = 0;
        shape->num_nodes = 0;
        if (root_box)
            for (int k = 0; k < 6; ++k) root_box[k] = 0.0f;
        return PIERCE_OK;
    }
    // scratch: 1 centroids, 2 keys (in|out), 3 vals (in|out), 4 leaf records + bounds
    void *pc = nullptr, *pk = nullptr, *pv = nullptr, *pm = nullptr;
    if (int s = scratch(ctx, 1, sizeof(float4) * (size_t)n, &pc)) return s;
    const size_t key_bytes = parts ? sizeof(uint64_t) : sizeof(uint32_t);
    if (int s = scratch(ctx, 2, 2 * key_bytes * (size_t)n, &pk)) return s;
    if (int s = scratch(ctx, 3, 2 * sizeof(uint32_t) * (size_t)n, &pv)) return s;
    const size_t part_bounds = parts ? 24 * (size_t)num_parts : 0;
    if (int s = scratch(ctx, 4, sizeof(unsigned long long) * (size_t)n + 64 + 64 + part_bounds, &pm)) return s;
    float4* cen = static_cast<float4*>(pc);
    uint32_t* keys = static_cast<uint32_t*>(pk);
    uint32_t* vals = static_cast<uint32_t*>(pv);
    unsigned long long* leaf_rec = static_cast<unsigned long long*>(pm);
    uint32_t* bounds = reinterpret_cast<uint32_t*>(leaf_rec + n);  // 6 words
    float* d_root_box = reinterpret_cast<float*>(bounds + 6);        // 6 floats
    // byte layout after the n leaf records: bounds [8n, 8n+24), root box
    // [8n+24, 8n+48), two wave counters [8n+64, 8n+80); allocation 8n+128
    unsigned long long* wave_count = leaf_rec + n + 8;
    // partitioned: per-partition bounds after that, [8n+128, ...)
    uint32_t* pbounds = reinterpret_cast<uint32_t*>(leaf_rec + n + 16);
    uint64_t* keys64 = static_cast<uint64_t*>(pk);

    const int B = 256;
    if (parts) {
        const int64_t nb = 6 * (int64_t)num_parts;
        k_obj_box_init<<<grid_for(ctx, nb, B), B, 0, st>>>(pbounds, num_parts);  // ordered (+max, -max)
        k_centroids_parts<<<grid_for(ctx, n, B), B, 0, st>>>(verts, idx, list, t2o, obj_part, n, cen, pbounds);
        k_morton_parts<<<grid_for(ctx, n, B), B, 0, st>>>(cen, n, pbounds, keys64, vals);
        ctx->launches += 3;
        int bits = 0;
        while (bits < 32 && (1ll << bits) < (int64_t)num_parts) ++bits;
        if (int s = sort_u64_pairs(ctx, keys64, keys64 + n, vals, vals + n, n, 30 + bits)) return s;
    } else {
        k_fill_u32<<<1, 32, 0, st>>>(bounds, 0xFFFFFFFFu, 3);  // ordered +max
        k_fill_u32<<<1, 32, 0, st>>>(bounds + 3, 0u, 3);       // ordered -max
        k_centroids<<<std::min(grid_for(ctx, n, B), ctx->sm_count * 4), B, 0, st>>>(verts, idx, list, n, cen, bounds);
        k_morton<<<grid_for(ctx, n, B), B, 0, st>>>(cen, n, bounds, keys, vals);
        ctx->launches += 4;
        if (int s = sort_u32_pairs(ctx, keys, keys + n, vals, vals + n, n, 30)) return s;
    }
    const uint32_t* skeys = keys + n;
    const uint64_t* skeys64 = keys64 + n;
    const uint32_t* order = vals + n;
    k_soup<<<grid_for(ctx, n, B), B, 0, st>>>(verts, idx, t2o, list, order, n, soup);
    ctx->launches += 1;
    // a partitioned hierarchy keeps an internal root unless it holds one
    // triangle: a root leaf could mix partitions
    if (parts ? n == 1 : n <= leaf_size) {
        k_single_box<<<1, 1, 0, st>>>(soup, n, d_root_box);
        ctx->launches += 1;
        if (parts) {
            k_single_part_root<<<1, 1, 0, st>>>(skeys64, part_roots);
            ctx->launches += 1;
        }
        shape->root_is_leaf = 1;
        shape->root_leaf_count = (int)n;
        shape->num_nodes = 0;
    } else {
        cudaMemsetAsync(leaf_rec, 0xFF, sizeof(unsigned long long) * (size_t)n, st);
        if (parts)
            k_karras<uint64_t><<<grid_for(ctx, n - 1, B), B, 0, st>>>(skeys64, n, leaf_size, nodes, leaf_rec,
                                                                      part_roots);
        else
            k_karras<uint32_t><<<grid_for(ctx, n - 1, B), B, 0, st>>>(skeys, n, leaf_size, nodes, leaf_rec,
                                                                      nullptr);
        // waves for the wide bottom levels, then one chain launch for the rest;
        // the lists reuse the Morton key buffer (free after the hierarchy step)
        uint32_t* lists[2] = {keys, keys + (n + 1) / 2 + 1};
        cudaMemsetAsync(wave_count, 0, 2 * sizeof(unsigned long long), st);
        k_refit_leaves<<<grid_for(ctx, n, B), B, 0, st>>>(soup, n, nodes, leaf_rec, lists[0], wave_count);
        // small hierarchies (object and chunk boxes) go straight to the chain:
        // their waves would be launches of a few blocks each
        const int kWaves = n >= (1 << 18) ? 3 : 0;
        for (int wave = 0; wave < kWaves; ++wave) {
            const int in = wave & 1, out = in ^ 1;
            cudaMemsetAsync(wave_count + out, 0, sizeof(unsigned long long), st);
            k_refit_wave<<<grid_for(ctx, n / 2 + 1, B), B, 0, st>>>(nodes, n - 1, lists[in], wave_count + in,
                                                                       n / 2 + 1, lists[out], wave_count + out,
                                                                       d_root_box);
        }
        const int last = kWaves & 1;
        k_refit_chain<<<grid_for(ctx, n / 2 + 1, B), B, 0, st>>>(nodes, n - 1, lists[last], wave_count + last,
                                                                    n / 2 + 1, d_root_box, ctx->d_err);
        ctx->launches += 3 + kWaves;
        shape->num_nodes = (uint64_t)(n - 1);
        shape->root_is_leaf = 0;
        shape->root_leaf_count = 0;
    }
    if (int s = check_cuda(cudaGetLastError(), "bvh build kernels")) return s;
    if (root_box) {
        if (int s = check_cuda(cudaMemcpyAsync(root_box, d_root_box, 6 * sizeof(float), cudaMemcpyDeviceToHost, st),
                               "bvh root box"))
            return s;
        if (int s = check_cuda(cudaStreamSynchronize(st), "bvh build")) return s;
    }
    return PIERCE_OK;
}

// ---- hierarchies over groups of consecutive triangles --------------------
// The per-join hierarchies are built over the chunks that survive culling.
// Consecutive triangles of a mesh lie close together, so a group of G of
// them (G divides 32) makes a tight leaf by itself: the hierarchy is built
// over the group boxes (32/G per active 32-triangle chunk) instead of over
// single triangles, which sorts and links G times fewer primitives; the
// triangle soup then takes the groups in leaf order, G triangles per leaf.

// Per listed chunk, the boxes of its groups as degenerate triangles
// (lo, hi, hi).  Triangles past the end of the dataset (final partial chunk)
// repeat the chunk's first triangle.
// Triangle k of group j of chunk c.  Past the last triangle a group repeats
// its own first triangle (or, when it has none, the chunk's first), so a
// group never mixes objects that its real triangles do not.
__device__ __forceinline__ int64_t group_item(int64_t c, int j, int G, int k, int64_t nt) {
    const int64_t first = c * 32 + (int64_t)j * G;
    const int64_t t = first + k;
    if (t < nt) return t;
    return first < nt ? first : c * 32;
}

__global__ void __launch_bounds__(256) k_group_boxes(const float* __restrict__ verts, const uint32_t* __restrict__ idx,
                                                     const int32_t* __restrict__ t2o, int64_t nt,
                                                     const uint32_t* __restrict__ chunk_list, int64_t n_chunks,
                                                     int G, float* __restrict__ gbox, uint32_t* __restrict__ gidx,
                                                     int32_t* __restrict__ gt2o) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t k = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < n_chunks; k += warps) {
        const int64_t c = chunk_list[k];
        int64_t t = group_item(c, lane / G, G, lane % G, nt);
        float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
        for (int v = 0; v < 3; ++v) {
            const float3 p = load_vertex(verts, __ldg(idx + 3 * t + v));
            lo[0] = fminf(lo[0], p.x); lo[1] = fminf(lo[1], p.y); lo[2] = fminf(lo[2], p.z);
            hi[0] = fmaxf(hi[0], p.x); hi[1] = fmaxf(hi[1], p.y); hi[2] = fmaxf(hi[2], p.z);
        }
        for (int off = 1; off < G; off <<= 1)
            for (int d = 0; d < 3; ++d) {
                lo[d] = fminf(lo[d], __shfl_xor_sync(0xFFFFFFFFu, lo[d], off));
                hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xFFFFFFFFu, hi[d], off));
            }
        if (lane % G == 0) {
            const int64_t g = k * (32 / G) + lane / G;
            float* b = gbox + 6 * g;
            b[0] = lo[0]; b[1] = lo[1]; b[2] = lo[2];
            b[3] = hi[0]; b[4] = hi[1]; b[5] = hi[2];
            gidx[3 * g] = (uint32_t)(2 * g);
            gidx[3 * g + 1] = (uint32_t)(2 * g + 1);
            gidx[3 * g + 2] = (uint32_t)(2 * g + 1);
            gt2o[g] = __ldg(t2o + t);
        }
    }
}

// Triangle soup in group leaf order: leaf position j takes group g (its
// original index, stored by k_soup in the group soup), G triangles each.
__global__ void __launch_bounds__(256) k_group_soup(const float4* __restrict__ gsoup, int64_t n_groups, int G,
                                                    const uint32_t* __restrict__ chunk_list,
                                                    const float* __restrict__ verts, const uint32_t* __restrict__ idx,
                                                    const int32_t* __restrict__ t2o, int64_t nt,
                                                    float4* __restrict__ soup) {
    const int per_chunk = 32 / G;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_groups * G;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = i / G;
        const int64_t g = __float_as_int(__ldg(&gsoup[3 * j + 1].w));
        const int64_t c = chunk_list[g / per_chunk];
        const int64_t t = group_item(c, (int)(g % per_chunk), G, (int)(i % G), nt);
        const float3 a = load_vertex(verts, __ldg(idx + 3 * t));
        const float3 b = load_vertex(verts, __ldg(idx + 3 * t + 1));
        const float3 cc = load_vertex(verts, __ldg(idx + 3 * t + 2));
        soup[3 * i + 0] = make_float4(a.x, a.y, a.z, __int_as_float(__ldg(t2o + t)));
        soup[3 * i + 1] = make_float4(b.x, b.y, b.z, __int_as_float((int)t));
        soup[3 * i + 2] = make_float4(cc.x, cc.y, cc.z, 0.0f);
    }
}

// Leaves of the group hierarchy (one group each) become soup ranges of G.
__global__ void k_group_leaves(Node* nodes, int64_t num_nodes, int G) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < num_nodes; i += (int64_t)gridDim.x * blockDim.x) {
        int4 ch = nodes[i].ch;
        int c0 = ch.z & 0xFF, c1 = (ch.z >> 8) & 0xFF;
        if (ch.x < 0) {
            ch.x = ~((~ch.x) * G);
            c0 = G;
        }
        if (ch.y < 0) {
            ch.y = ~((~ch.y) * G);
            c1 = G;
        }
        ch.z = c0 | (c1 << 8);
        nodes[i].ch = ch;
    }
}

// One thread per binary internal node: entries 0-1 come from child 0 and
// 2-3 from child 1 -- the child's own two children when it is internal, the
// child itself (and an empty entry) when it is a leaf.  With leaf sizes
// above one, the internal nodes inside a collapsed leaf are never written by
// the build and hold stale values: a child index outside [0, n) is not
// followed (it only occurs in such unreachable nodes, whose Node4 copies are
// never read).
__device__ __forceinline__ void node4_half(const Node* __restrict__ nodes, int64_t n, const float4& bx,
                                           const float4& by, const float4& bz, const int4& c, int side,
                                           float (&lo)[3][2], float (&hi)[3][2], int (&ch)[2], int (&cnt)[2]) {
    const int r = side ? c.y : c.x;
    if (r >= 0 && (int64_t)r >= n) {
        for (int j = 0; j < 2; ++j) {
            for (int k = 0; k < 3; ++k) {
                lo[k][j] = 3.4e38f;
                hi[k][j] = -3.4e38f;
            }
            ch[j] = -1;
            cnt[j] = 0;
        }
        return;
    }
    if (r < 0) {
        lo[0][0] = side ? bx.z : bx.x; hi[0][0] = side ? bx.w : bx.y;
        lo[1][0] = side ? by.z : by.x; hi[1][0] = side ? by.w : by.y;
        lo[2][0] = side ? bz.z : bz.x; hi[2][0] = side ? bz.w : bz.y;
        ch[0] = r;
        cnt[0] = (c.z >> (8 * side)) & 0xFF;
        for (int k = 0; k < 3; ++k) {
            lo[k][1] = 3.4e38f;
            hi[k][1] = -3.4e38f;
        }
        ch[1] = -1;
        cnt[1] = 0;
        return;
    }
    const float4 gx = __ldg(&nodes[r].bx), gy = __ldg(&nodes[r].by), gz = __ldg(&nodes[r].bz);
    const int4 gc = __ldg(&nodes[r].ch);
    lo[0][0] = gx.x; hi[0][0] = gx.y; lo[0][1] = gx.z; hi[0][1] = gx.w;
    lo[1][0] = gy.x; hi[1][0] = gy.y; lo[1][1] = gy.z; hi[1][1] = gy.w;
    lo[2][0] = gz.x; hi[2][0] = gz.y; lo[2][1] = gz.z; hi[2][1] = gz.w;
    ch[0] = gc.x;
    ch[1] = gc.y;
    cnt[0] = gc.z & 0xFF;
    cnt[1] = (gc.z >> 8) & 0xFF;
}

__global__ void __launch_bounds__(256) k_collapse4(const Node* __restrict__ nodes, int64_t n, Node4* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 bx = __ldg(&nodes[i].bx), by = __ldg(&nodes[i].by), bz = __ldg(&nodes[i].bz);
        const int4 c = __ldg(&nodes[i].ch);
        float lo0[3][2], hi0[3][2], lo1[3][2], hi1[3][2];
        int ch0[2], ch1[2], n0[2], n1[2];
        node4_half(nodes, n, bx, by, bz, c, 0, lo0, hi0, ch0, n0);
        node4_half(nodes, n, bx, by, bz, c, 1, lo1, hi1, ch1, n1);
        Node4 q;
        q.lox = make_float4(lo0[0][0], lo0[0][1], lo1[0][0], lo1[0][1]);
        q.hix = make_float4(hi0[0][0], hi0[0][1], hi1[0][0], hi1[0][1]);
        q.loy = make_float4(lo0[1][0], lo0[1][1], lo1[1][0], lo1[1][1]);
        q.hiy = make_float4(hi0[1][0], hi0[1][1], hi1[1][0], hi1[1][1]);
        q.loz = make_float4(lo0[2][0], lo0[2][1], lo1[2][0], lo1[2][1]);
        q.hiz = make_float4(hi0[2][0], hi0[2][1], hi1[2][0], hi1[2][1]);
        q.ch = make_int4(ch0[0], ch0[1], ch1[0], ch1[1]);
        q.meta = make_int4(n0[0] | (n0[1] << 8) | (n1[0] << 16) | (n1[1] << 24), 0, 0, 0);
        out[i] = q;
    }
}

int collapse4(pierce_ctx* ctx, const Node* nodes, int64_t num_nodes, Node4* out) {
    if (num_nodes <= 0) return PIERCE_OK;
    k_collapse4<<<grid_for(ctx, num_nodes, 256), 256, 0, ctx->stream>>>(nodes, num_nodes, out);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "collapse to four-wide nodes");
}

// Partitioned datasets: does any group of G triangles of a flagged chunk
// (every chunk when chunk_flags is null) hold triangles of two partitions?
// (Then the join builds over triangles.)
__global__ void __launch_bounds__(256) k_group_mixed(const uint8_t* __restrict__ chunk_flags, int64_t n_chunks,
                                                     const int32_t* __restrict__ t2o,
                                                     const int32_t* __restrict__ obj_part, int64_t nt, int G,
                                                     int32_t* mixed) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t c = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < n_chunks; c += warps) {
        if (chunk_flags && !chunk_flags[c]) continue;  // warp-uniform
        const int64_t t = group_item(c, lane / G, G, lane % G, nt);
        const int32_t o = __ldg(t2o + t);
        const int32_t p = o >= 0 ? __ldg(obj_part + o) : -1;
        const int32_t p0 = __shfl_sync(0xFFFFFFFFu, p, lane & ~(G - 1));
        if (__any_sync(0xFFFFFFFFu, p != p0) && lane == 0) atomicOr(mixed, 1);
    }
}

int launch_group_mixed(pierce_ctx* ctx, const uint8_t* chunk_flags, int64_t n_chunks, const int32_t* t2o,
                       const int32_t* obj_part, int64_t nt, int G, int32_t* mixed) {
    if (n_chunks <= 0) return PIERCE_OK;
    k_group_mixed<<<grid_for(ctx, n_chunks * 32, 256), 256, 0, ctx->stream>>>(chunk_flags, n_chunks, t2o, obj_part,
                                                                             nt, G, mixed);
    ctx->launches += 1;
    return check_cuda(cudaGetLastError(), "group partition check");
}

// Partition roots of a group hierarchy: a root leaf of one group becomes the
// soup range of its G triangles.
__global__ void k_group_roots(int2* roots, int32_t num_parts, int G) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < num_parts;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int2 r = roots[p];
        if (r.x < 0 && r.y > 0) roots[p] = make_int2(~((~r.x) * G), r.y * G);
    }
}

int build_grouped_lbvh(pierce_ctx* ctx, const float* verts, const uint32_t* idx, const int32_t* t2o, int64_t nt,
                       const uint32_t* chunk_list, int64_t n_chunks, int G, void* group_scratch, float4* soup,
                       Node* nodes, BvhShape* shape, const DevDataset* filter, unsigned long long* d_count,
                       int64_t* kept, const int32_t* obj_part, int32_t num_parts, int2* part_roots) {
    cudaStream_t st = ctx->stream;
    const int64_t ng = n_chunks * (32 / G);
    shape->leaf_size = G;
    const bool parts = obj_part && num_parts > 0 && part_roots;
    if (ng == 0) {
        shape->root_is_leaf = 1;
        shape->root_leaf_count = 0;
        shape->num_nodes = 0;
        if (kept) *kept = 0;
        if (parts) {
            k_fill_roots<<<grid_for(ctx, num_parts, 256), 256, 0, st>>>(part_roots, num_parts);
            ctx->launches += 1;
        }
        return check_cuda(cudaGetLastError(), "grouped bvh build");
    }
    if (ng * G >= (int64_t(1) << 30))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "bvh build: at most 2^30 - 1 triangles per hierarchy");
    // group scratch: soup 48, boxes 24, pseudo indices 12, ids 4, filter flags 1
    // and kept-group list 4 bytes per group
    char* q = static_cast<char*>(group_scratch);
    float4* gsoup = reinterpret_cast<float4*>(q);
    float* gbox = reinterpret_cast<float*>(q + 48 * ng);
    uint32_t* gidx = reinterpret_cast<uint32_t*>(q + 72 * ng);
    int32_t* gt2o = reinterpret_cast<int32_t*>(q + 84 * ng);
    const int64_t warps = n_chunks;
    k_group_boxes<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((warps + 7) / 8, (int64_t)ctx->sm_count * 16)),
                    256, 0, st>>>(verts, idx, t2o, nt, chunk_list, n_chunks, G, gbox, gidx, gt2o);
    ctx->launches += 1;
    // optional filter: keep the groups that can meet the other side
    const uint32_t* list = nullptr;
    int64_t n = ng;
    if (filter) {
        uint8_t* flags = reinterpret_cast<uint8_t*>(q + 88 * ng);
        char* lq = q + 88 * ng + ng;
        lq += (256 - ((uintptr_t)lq & 255)) & 255;
        uint32_t* glist = reinterpret_cast<uint32_t*>(lq);
        if (int s = launch_group_filter(ctx, gbox, ng, *filter, parts ? gt2o : nullptr, obj_part, flags)) return s;
        if (int s = select_flagged(ctx, flags, ng, glist, d_count)) return s;
        if (int s = host_value(ctx, d_count, 8, &n, "kept groups")) return s;
        list = glist;
    }
    if (kept) *kept = n;
    if (n == 0) {
        shape->root_is_leaf = 1;
        shape->root_leaf_count = 0;
        shape->num_nodes = 0;
        if (parts) {
            k_fill_roots<<<grid_for(ctx, num_parts, 256), 256, 0, st>>>(part_roots, num_parts);
            ctx->launches += 1;
        }
        return check_cuda(cudaGetLastError(), "grouped bvh build");
    }
    BvhShape gshape;
    if (int s = build_lbvh(ctx, gbox, gidx, gt2o, list, n, 1, gsoup, nodes, &gshape, nullptr,
                           parts ? obj_part : nullptr, parts ? num_parts : 0, parts ? part_roots : nullptr))
        return s;
    k_group_soup<<<grid_for(ctx, n * G, 256), 256, 0, st>>>(gsoup, n, G, chunk_list, verts, idx, t2o, nt, soup);
    ctx->launches += 1;
    if (gshape.root_is_leaf) {
        shape->root_is_leaf = 1;
        shape->root_leaf_count = (int)(gshape.root_leaf_count * G);
        shape->num_nodes = 0;
    } else {
        k_group_leaves<<<grid_for(ctx, (int64_t)gshape.num_nodes, 256), 256, 0, st>>>(nodes,
                                                                                     (int64_t)gshape.num_nodes, G);
        ctx->launches += 1;
    }
    if (parts) {
        k_group_roots<<<grid_for(ctx, num_parts, 256), 256, 0, st>>>(part_roots, num_parts, G);
        ctx->launches += 1;
    }
    if (!gshape.root_is_leaf) {
        shape->root_is_leaf = 0;
        shape->root_leaf_count = 0;
        shape->num_nodes = gshape.num_nodes;
    }
    return check_cuda(cudaGetLastError(), "grouped bvh build");
}

int build_bvh(pierce_ctx* ctx, pierce_dataset* ds, int leaf_size) {
    ds->built = 0;
    // The soup and node arrays exist only for datasets that get a hierarchy
    // of their own (joins with per-join hierarchies never need them).
    if (!ds->d_soup) {
        if (int s = dataset_array(ctx, (void**)&ds->d_soup, 48 * std::max<uint64_t>(ds->nt, 1), ctx->stream,
                                  "triangle soup"))
            return s;
        ds->device_bytes += 48 * ds->nt;
    }
    if (!ds->d_nodes) {
        if (int s = dataset_array(ctx, (void**)&ds->d_nodes, sizeof(Node) * std::max<uint64_t>(ds->nt, 1), ctx->stream,
                                  "bvh nodes"))
            return s;
        ds->device_bytes += sizeof(Node) * ds->nt;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    BvhShape shape;
    float root_box[6] = {0, 0, 0, 0, 0, 0};
    int status = build_lbvh(ctx, ds->d_vertices, ds->d_indices, ds->d_tri_to_object, nullptr, (int64_t)ds->nt,
                            leaf_size, ds->d_soup, ds->d_nodes, &shape, root_box, ds->d_obj_part, ds->num_parts,
                            ds->d_part_roots);
    cudaEventRecord(e1, ctx->stream);
    if (status == PIERCE_OK) status = check_cuda(cudaStreamSynchronize(ctx->stream), "bvh build");
    float ms = 0.0f;
    if (status == PIERCE_OK) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (status != PIERCE_OK) return status;
    ds->leaf_size = shape.leaf_size;
    ds->root_is_leaf = shape.root_is_leaf;
    ds->root_leaf_count = shape.root_leaf_count;
    ds->num_nodes = shape.num_nodes;
    for (int k = 0; k < 3; ++k) {
        ds->lo[k] = root_box[k];
        ds->hi[k] = root_box[3 + k];
    }
    ds->ms_build = ms;
    ds->built = 1;
    return PIERCE_OK;
}

}  // namespace pgpu
