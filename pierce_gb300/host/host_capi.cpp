// C entry points of the host library (include/pierce_host.h).
#include <cstring>
#include <memory>
#include <string>

#include "geometry.h"

namespace {
thread_local std::string g_last_error;
}

namespace pierce {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace pierce

extern "C" const char* pierce_host_last_error(void) { return g_last_error.c_str(); }

extern "C" int pierce_geom_create(const float* vertices, uint64_t num_vertices, const uint32_t* indices,
                                  uint64_t num_triangles, const int32_t* tri_to_object, pierce_geom** out) {
    if (!out || (num_vertices && !vertices) || (num_triangles && (!indices || !tri_to_object))) {
        pierce::set_last_error("geom_create: null argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    std::unique_ptr<pierce_geom> g(new pierce_geom());
    g->vertices.assign(vertices, vertices + 3 * num_vertices);
    g->indices.assign(indices, indices + 3 * num_triangles);
    g->tri_to_object.assign(tri_to_object, tri_to_object + num_triangles);
    g->total_triangles = num_triangles;
    *out = g.release();
    return PIERCE_HOST_OK;
}

extern "C" void pierce_geom_free(pierce_geom* g) { delete g; }

extern "C" int pierce_geom_get_view(const pierce_geom* g, pierce_geom_view* v) {
    if (!g || !v) {
        pierce::set_last_error("geom_get_view: null argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    std::memset(v, 0, sizeof(*v));
    v->vertices = g->vertices.data();
    v->num_vertices = g->num_vertices();
    v->indices = g->indices.data();
    v->num_triangles = g->num_triangles();
    v->tri_to_object = g->tri_to_object.data();
    v->num_mappings = g->tri_to_object.size();
    v->total_triangles = g->total_triangles;
    v->edge_starts = g->edge_starts.data();
    v->edge_ends = g->edge_ends.data();
    v->edge_src = g->edge_src.data();
    v->num_edges = g->num_edges();
    v->has_edges = g->has_edges() ? 1 : 0;
    v->has_grid = g->has_grid ? 1 : 0;
    v->grid_cell_size = g->grid_cell_size;
    v->num_grid_cells = (uint32_t)g->grid_cells.size();
    v->grid_cells = g->grid_cells.data();
    v->num_objects = g->num_objects();
    return PIERCE_HOST_OK;
}

extern "C" int pierce_geom_set_edges(pierce_geom* g, const float* starts, const float* ends, const int32_t* src,
                                     uint64_t num_edges) {
    if (!g || (num_edges && (!starts || !ends || !src))) {
        pierce::set_last_error("geom_set_edges: null argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    g->edge_starts.assign(starts, starts + 3 * num_edges);
    g->edge_ends.assign(ends, ends + 3 * num_edges);
    g->edge_src.assign(src, src + num_edges);
    return PIERCE_HOST_OK;
}

extern "C" int pierce_geom_extract_edges(pierce_geom* g, int order, int num_threads) {
    if (!g || (order != 0 && order != 1)) {
        pierce::set_last_error("geom_extract_edges: invalid argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    pierce::extract_edges(*g, order, num_threads);
    return PIERCE_HOST_OK;
}

extern "C" int pierce_geom_grid_stats(pierce_geom* g, float cell_size) {
    if (!g || !(cell_size > 0.0f)) {
        pierce::set_last_error("geom_grid_stats: invalid argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    pierce::grid_stats(*g, cell_size);
    return PIERCE_HOST_OK;
}

extern "C" int pierce_geom_first_vertices(const pierce_geom* g, float* out, int32_t num_objects) {
    if (!g || (num_objects > 0 && !out)) {
        pierce::set_last_error("geom_first_vertices: invalid argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    std::vector<char> seen((size_t)(num_objects > 0 ? num_objects : 0), 0);
    for (int32_t i = 0; i < 3 * num_objects; ++i) out[i] = 0.0f;
    const uint64_t nt = g->num_triangles(), nv = g->num_vertices();
    for (uint64_t t = 0; t < nt && t < g->tri_to_object.size(); ++t) {
        const int32_t o = g->tri_to_object[t];
        if (o < 0 || o >= num_objects || seen[o]) continue;
        const uint32_t vi = g->indices[3 * t];
        if (vi >= nv) continue;
        std::memcpy(&out[3 * (size_t)o], &g->vertices[3 * (size_t)vi], 3 * sizeof(float));
        seen[o] = 1;
    }
    return PIERCE_HOST_OK;
}

extern "C" int pierce_geom_append(pierce_geom* a, const pierce_geom* b) {
    if (!a || !b) {
        pierce::set_last_error("geom_append: null argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    const uint32_t vbase = (uint32_t)a->num_vertices();
    const int32_t obase = a->num_objects();
    a->vertices.insert(a->vertices.end(), b->vertices.begin(), b->vertices.end());
    for (uint32_t i : b->indices) a->indices.push_back(vbase + i);
    for (int32_t o : b->tri_to_object) a->tri_to_object.push_back(o + obase);
    a->total_triangles = a->num_triangles();
    a->edge_starts.insert(a->edge_starts.end(), b->edge_starts.begin(), b->edge_starts.end());
    a->edge_ends.insert(a->edge_ends.end(), b->edge_ends.begin(), b->edge_ends.end());
    for (int32_t o : b->edge_src) a->edge_src.push_back(o + obase);
    a->has_grid = false;
    a->grid_cells.clear();
    return PIERCE_HOST_OK;
}
