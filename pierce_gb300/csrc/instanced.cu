// Device expansion of instanced icosphere datasets.
//
// A generated workload of N meshes is described on the host by N
// pierce_mesh_instance records (168 bytes each); the vertices, triangles,
// triangle-to-object map and unique edges (the rays of the join) are written
// here directly into the dataset's device arrays, so a dataset of 10^8
// triangles costs a few milliseconds instead of a host generation pass and a
// multi-gigabyte upload.  The vertex arithmetic is pierce::inst::instance_vertex
// (host/instance_math.h), evaluated with round-to-nearest double intrinsics,
// which makes the result bit-identical to the host expansion
// pierce_expand_instances in libpierce_host.
//
// Layout: mesh m occupies the contiguous ranges [voff[m], voff[m+1]) of
// vertices, [toff[m], toff[m+1]) of triangles and [eoff[m], eoff[m+1]) of
// edges, in mesh order; its object id is m.  Edges follow the template's
// unique-edge order (first-seen orientation over the template triangles).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "../host/icosphere.h"
#include "../host/instance_math.h"
#include "common.cuh"

namespace {

using pierce::inst::template_edges;
using pierce::inst::template_triangles;
using pierce::inst::template_vertices;

constexpr int kLevels = PIERCE_MAX_INSTANCE_LEVEL + 1;

struct TemplateSet {
    const double* verts[kLevels];    // 3 doubles per vertex
    const uint32_t* tris[kLevels];   // 3 per triangle
    const uint32_t* edges[kLevels];  // 2 per edge
};

using HostTemplate = pierce::inst::IcoTemplate;

// Index of the mesh whose range [off[m], off[m+1]) holds item i.
__device__ __forceinline__ int32_t find_mesh(const int64_t* __restrict__ off, int32_t n, int64_t i) {
    int32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const int32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void k_inst_vertices(const pierce_mesh_instance* __restrict__ inst, const int64_t* __restrict__ voff,
                                int32_t n, TemplateSet ts, float* __restrict__ out, int64_t nv) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t m = find_mesh(voff, n, i);
        const pierce_mesh_instance p = inst[m];
        const double* u = ts.verts[p.level] + 3 * (i - voff[m]);
        float w[3];
        pierce::inst::instance_vertex(p, u[0], u[1], u[2], w);
        out[3 * i] = w[0];
        out[3 * i + 1] = w[1];
        out[3 * i + 2] = w[2];
    }
}

__global__ void k_inst_triangles(const pierce_mesh_instance* __restrict__ inst, const int64_t* __restrict__ voff,
                                 const int64_t* __restrict__ toff, int32_t n, TemplateSet ts,
                                 uint32_t* __restrict__ idx, int32_t* __restrict__ t2o, int64_t nt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nt; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t m = find_mesh(toff, n, i);
        const uint32_t* t = ts.tris[inst[m].level] + 3 * (i - toff[m]);
        const uint32_t base = (uint32_t)voff[m];
        idx[3 * i] = base + t[0];
        idx[3 * i + 1] = base + t[1];
        idx[3 * i + 2] = base + t[2];
        t2o[i] = m;
    }
}

__global__ void k_inst_edges(const pierce_mesh_instance* __restrict__ inst, const int64_t* __restrict__ voff,
                             const int64_t* __restrict__ eoff, int32_t n, TemplateSet ts,
                             const float* __restrict__ verts, float4* __restrict__ edges,
                             int32_t* __restrict__ edge_src, int64_t ne) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ne; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t m = find_mesh(eoff, n, i);
        const uint32_t* e = ts.edges[inst[m].level] + 2 * (i - eoff[m]);
        const float* a = verts + 3 * (voff[m] + e[0]);
        const float* b = verts + 3 * (voff[m] + e[1]);
        edges[2 * i] = make_float4(a[0], a[1], a[2], __int_as_float(m));
        edges[2 * i + 1] = make_float4(b[0], b[1], b[2], 0.0f);
        edge_src[i] = m;
    }
}

int grid_for(pierce_ctx* ctx, int64_t n, int block) {
    int64_t b = (n + block - 1) / block;
    const int64_t cap = (int64_t)ctx->sm_count * 16;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace

using namespace pgpu;

extern "C" int pierce_dataset_create_instanced(pierce_ctx* ctx, const pierce_mesh_instance* meshes,
                                               int32_t num_meshes, const pierce_tuning* tuning,
                                               pierce_dataset** out) {
    if (!ctx || !out || (!meshes && num_meshes) || num_meshes < 0)
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "dataset_create_instanced: invalid argument");
    *out = nullptr;
    // Per-mesh offsets and the template levels in use.
    std::vector<int64_t> off(3 * ((size_t)num_meshes + 1));
    int64_t* voff = off.data();
    int64_t* toff = voff + num_meshes + 1;
    int64_t* eoff = toff + num_meshes + 1;
    bool used[kLevels] = {false};
    int32_t max_group = 0;
    for (int32_t m = 0; m < num_meshes; ++m) {
        const int l = meshes[m].level;
        if (meshes[m].group < 0)
            return set_error(PIERCE_ERR_INVALID_ARGUMENT, "dataset_create_instanced: negative group");
        max_group = std::max(max_group, meshes[m].group);
        if (l < 0 || l >= kLevels)
            return set_error(PIERCE_ERR_INVALID_ARGUMENT, "dataset_create_instanced: level out of range");
        used[l] = true;
        voff[m + 1] = voff[m] + template_vertices(l);
        toff[m + 1] = toff[m] + template_triangles(l);
        eoff[m + 1] = eoff[m] + template_edges(l);
    }
    const uint64_t nv = (uint64_t)voff[num_meshes], nt = (uint64_t)toff[num_meshes], ne = (uint64_t)eoff[num_meshes];
    if (nt >= (1ull << 31) || nv >= (1ull << 32))
        return set_error(PIERCE_ERR_INVALID_ARGUMENT, "dataset_create_instanced: dataset too large for 32-bit ids");

    // Template blob: per used level doubles (vertices) then uint32 (tris, edges).
    std::vector<HostTemplate> tmpl(kLevels);
    size_t blob_bytes = 0;
    size_t v_at[kLevels] = {0}, t_at[kLevels] = {0}, e_at[kLevels] = {0};
    for (int l = 0; l < kLevels; ++l) {
        if (!used[l]) continue;
        tmpl[l] = pierce::inst::make_icosphere_template(l);
        v_at[l] = blob_bytes;
        blob_bytes += 8 * tmpl[l].v.size();
        t_at[l] = blob_bytes;
        blob_bytes += 4 * tmpl[l].t.size();
        e_at[l] = blob_bytes;
        blob_bytes += 4 * tmpl[l].e.size();
        blob_bytes = (blob_bytes + 15) & ~size_t(15);
    }
    std::vector<unsigned char> blob(std::max<size_t>(blob_bytes, 16));
    for (int l = 0; l < kLevels; ++l) {
        if (!used[l]) continue;
        std::copy_n(reinterpret_cast<const unsigned char*>(tmpl[l].v.data()), 8 * tmpl[l].v.size(), &blob[v_at[l]]);
        std::copy_n(reinterpret_cast<const unsigned char*>(tmpl[l].t.data()), 4 * tmpl[l].t.size(), &blob[t_at[l]]);
        std::copy_n(reinterpret_cast<const unsigned char*>(tmpl[l].e.data()), 4 * tmpl[l].e.size(), &blob[e_at[l]]);
    }

    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    pierce_dataset* ds = new pierce_dataset();
    ds->ctx = ctx;
    ds->device = ctx->device;
    ds->nv = nv;
    ds->nt = nt;
    ds->ne = (tuning && tuning->skip_edges) ? 0 : ne;  // skip_edges: rays come from the triangles
    ds->num_objects = num_meshes;
    void *d_blob = nullptr, *d_inst = nullptr, *d_off = nullptr;
    int s = PIERCE_OK;
    do {
        if ((s = dataset_alloc(ds, st))) break;
        if ((s = device_alloc(&d_blob, blob.size(), "instance templates"))) break;
        if ((s = device_alloc(&d_inst, sizeof(pierce_mesh_instance) * std::max(num_meshes, 1), "instances"))) break;
        if ((s = device_alloc(&d_off, 8 * off.size(), "instance offsets"))) break;
        if ((s = check_cuda(cudaMemcpyAsync(d_blob, blob.data(), blob.size(), cudaMemcpyHostToDevice, st),
                            "copy templates")))
            break;
        if (num_meshes &&
            (s = check_cuda(cudaMemcpyAsync(d_inst, meshes, sizeof(pierce_mesh_instance) * num_meshes,
                                            cudaMemcpyHostToDevice, st),
                            "copy instances")))
            break;
        if ((s = check_cuda(cudaMemcpyAsync(d_off, off.data(), 8 * off.size(), cudaMemcpyHostToDevice, st),
                            "copy offsets")))
            break;
        TemplateSet ts{};
        for (int l = 0; l < kLevels; ++l) {
            const unsigned char* b = static_cast<const unsigned char*>(d_blob);
            ts.verts[l] = used[l] ? reinterpret_cast<const double*>(b + v_at[l]) : nullptr;
            ts.tris[l] = used[l] ? reinterpret_cast<const uint32_t*>(b + t_at[l]) : nullptr;
            ts.edges[l] = used[l] ? reinterpret_cast<const uint32_t*>(b + e_at[l]) : nullptr;
        }
        const pierce_mesh_instance* di = static_cast<const pierce_mesh_instance*>(d_inst);
        const int64_t* dv = static_cast<const int64_t*>(d_off);
        const int64_t* dt = dv + num_meshes + 1;
        const int64_t* de = dt + num_meshes + 1;
        if (nv) {
            k_inst_vertices<<<grid_for(ctx, (int64_t)nv, 256), 256, 0, st>>>(di, dv, num_meshes, ts, ds->d_vertices,
                                                                            (int64_t)nv);
            k_inst_triangles<<<grid_for(ctx, (int64_t)nt, 256), 256, 0, st>>>(di, dv, dt, num_meshes, ts,
                                                                             ds->d_indices, ds->d_tri_to_object,
                                                                             (int64_t)nt);
            ctx->launches += 2;
            if (ds->ne) {
                k_inst_edges<<<grid_for(ctx, (int64_t)ne, 256), 256, 0, st>>>(di, dv, de, num_meshes, ts,
                                                                             ds->d_vertices, ds->d_edges,
                                                                             ds->d_edge_src, (int64_t)ne);
                ctx->launches += 1;
            }
            if ((s = check_cuda(cudaGetLastError(), "instance expansion"))) break;
        }
        if (max_group > 0) {
            // a batch of joins: the mesh groups partition the dataset
            std::vector<int32_t> part((size_t)num_meshes);
            for (int32_t m = 0; m < num_meshes; ++m) part[m] = meshes[m].group;
            pierce_tuning t;
            pierce_default_tuning(&t);
            if (tuning) t = *tuning;
            t.defer_build = 1;
            if ((s = dataset_finish(ctx, ds, &t))) break;
            if ((s = pierce_dataset_set_partitions(ctx, ds, part.data(), max_group + 1))) break;
            if (!(tuning && tuning->defer_build) && (s = build_bvh(ctx, ds, ds->leaf_size))) break;
        } else if ((s = dataset_finish(ctx, ds, tuning))) {
            break;
        }
    } while (0);
    cudaStreamSynchronize(st);
    for (void* p : {d_blob, d_inst, d_off})
        if (p) cudaFree(p);
    if (s) {
        pierce_dataset_destroy(ds);
        return s;
    }
    *out = ds;
    return PIERCE_OK;
}
