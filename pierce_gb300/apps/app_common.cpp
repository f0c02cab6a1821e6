#include "app_common.h"

#include <cmath>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <set>

HostDataset::~HostDataset() {
    if (geom) pierce_geom_free(geom);
}

bool load_dataset(const std::string& path, HostDataset& out) {
    std::cout << "=== Loading Preprocessed Geometry (Binary) ===" << std::endl;
    const int s = pierce_geom_read_pre(path.c_str(), &out.geom);
    if (s != PIERCE_HOST_OK) {
        std::cerr << "Error: " << pierce_host_last_error() << std::endl;
        out.geom = nullptr;
        return false;
    }
    pierce_geom_get_view(out.geom, &out.view);
    if (out.view.num_vertices == 0) return false;
    std::set<int32_t> ids(out.view.tri_to_object, out.view.tri_to_object + out.view.num_mappings);
    out.unique_objects = (int)ids.size();
    return true;
}

bool require_edges(const HostDataset& d, const std::string& path, const char* label) {
    if (d.view.has_edges) return true;
    std::cerr << "Error: " << label << " loaded from '" << path << "' does not contain precomputed edges."
              << std::endl;
    std::cerr << "Re-run pierce_preprocess to regenerate the .pre file with embedded edge payload." << std::endl;
    return false;
}

pierce_mesh_view mesh_view(const HostDataset& d) {
    pierce_mesh_view v{};
    v.vertices = d.view.vertices;
    v.num_vertices = d.view.num_vertices;
    v.indices = d.view.indices;
    v.num_triangles = d.view.num_triangles;
    v.tri_to_object = d.view.tri_to_object;
    v.edge_starts = d.view.edge_starts;
    v.edge_ends = d.view.edge_ends;
    v.edge_src = d.view.edge_src;
    v.num_edges = d.view.num_edges;
    v.num_objects = d.view.num_objects;
    return v;
}

void fail(const char* what, int status) {
    std::cerr << "Error: " << what << ": " << pierce_status_string(status) << ": " << pierce_last_error()
              << std::endl;
    std::exit(EXIT_FAILURE);
}

void upload(pierce_ctx* ctx, const HostDataset& h, GpuDataset& g) {
    pierce_mesh_view v = mesh_view(h);
    pierce_tuning t;
    pierce_default_tuning(&t);
    t.defer_build = 1;
    check(pierce_dataset_create(ctx, &v, PIERCE_HOST_MEMORY, &t, &g.ds), "upload");
}

void build_index(pierce_ctx* ctx, GpuDataset& g) {
    pierce_tuning t;
    pierce_default_tuning(&t);
    check(pierce_dataset_build(ctx, g.ds, &t), "build index");
}

static float weighted_avg(const pierce_grid_entry* c, uint32_t n, bool ratio) {
    double sum = 0.0;
    long long cnt = 0;
    for (uint32_t i = 0; i < n; ++i)
        if (c[i].touch_count > 0) {
            sum += (double)(ratio ? c[i].vol_ratio : c[i].avg_size_mean) * (double)c[i].touch_count;
            cnt += c[i].touch_count;
        }
    if (cnt == 0) return ratio ? 1.0f : 0.0f;
    return (float)(sum / cnt);
}

Estimate estimate_pairs(pierce_ctx* ctx, const HostDataset& a, const HostDataset& b, float epsilon, float gamma,
                        bool alpha_correction, bool verbose_mismatch) {
    Estimate e;
    if (!a.view.has_grid || !b.view.has_grid) return e;
    e.has_grid = true;
    if (std::fabs(a.view.grid_cell_size - b.view.grid_cell_size) > 1e-5f && verbose_mismatch)
        std::cerr << "Warning: Grid cell sizes mismatch (Mesh1: " << a.view.grid_cell_size
                  << ", Mesh2: " << b.view.grid_cell_size << "). Estimation may be invalid." << std::endl;
    int64_t est = 0;
    int32_t matched = 0;
    check(pierce_estimate_pairs(ctx, a.view.grid_cells, a.view.num_grid_cells, b.view.grid_cells,
                                b.view.num_grid_cells, a.view.grid_cell_size, epsilon, gamma, alpha_correction ? 1 : 0,
                                &e.raw, &est, &matched),
          "selectivity estimation");
    e.pairs = est;
    e.matched_cells = matched;
    e.avg_size[0] = weighted_avg(a.view.grid_cells, a.view.num_grid_cells, false);
    e.avg_size[1] = weighted_avg(b.view.grid_cells, b.view.num_grid_cells, false);
    e.avg_ratio[0] = weighted_avg(a.view.grid_cells, a.view.num_grid_cells, true);
    e.avg_ratio[1] = weighted_avg(b.view.grid_cells, b.view.num_grid_cells, true);
    e.eff_size[0] = e.avg_size[0] * std::cbrt(e.avg_ratio[0]);
    e.eff_size[1] = e.avg_size[1] * std::cbrt(e.avg_ratio[1]);
    const float cs = a.view.grid_cell_size;
    float cell_volume = cs * cs * cs;
    if (cell_volume < 1e-9f) cell_volume = 1e-9f;
    const float comb = e.eff_size[0] + e.eff_size[1];
    e.alpha = 1.0f;
    if (alpha_correction) {
        e.alpha = comb * comb * comb / cell_volume;
        if (e.alpha < 1.0f) e.alpha = 1.0f;
    }
    return e;
}

long long micros(double ms) { return (long long)std::llround(ms * 1000.0); }

void write_pairs_csv(const std::string& path, const char* header, const std::vector<pierce_pair>& pairs) {
    std::ofstream f(path);
    if (!f) {
        std::cerr << "Warning: Failed to open pairs output file: " << path << std::endl;
        return;
    }
    f << header << "\n";
    for (const auto& p : pairs) f << p.a << "," << p.b << "\n";
}

std::vector<pierce_pair> download(pierce_ctx* ctx, pierce_result* r) {
    uint64_t n = 0;
    pierce_result_count(r, &n);
    std::vector<pierce_pair> out(n);
    if (n) check(pierce_result_copy(ctx, r, out.data(), n), "download results");
    return out;
}
