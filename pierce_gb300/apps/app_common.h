// Shared pieces of the query executables: loading `.pre` files, device
// datasets, the grid selectivity estimate and hash sizing, CSV output.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pierce_capi.h"
#include "../../include/pierce_host.h"

struct HostDataset {
    pierce_geom* geom = nullptr;
    pierce_geom_view view{};
    int unique_objects = 0;  // number of distinct object ids (std::set size in the reference)
    ~HostDataset();
};

// loadGeometryFromFile + the caller's empty check
// (pierce/query/src/runtime/GeometryIO.cpp:6-9).  Prints the reference's
// messages; false on failure.
bool load_dataset(const std::string& path, HostDataset& out);
// requirePrecomputedEdges (GeometryIO.cpp:11-20).
bool require_edges(const HostDataset& d, const std::string& path, const char* label);

pierce_mesh_view mesh_view(const HostDataset& d);

// Abort the application with the library's last error (the library itself
// never exits).
[[noreturn]] void fail(const char* what, int status);
inline void check(int status, const char* what) {
    if (status != PIERCE_OK) fail(what, status);
}

struct GpuDataset {
    pierce_dataset* ds = nullptr;
    ~GpuDataset() {
        if (ds) pierce_dataset_destroy(ds);
    }
};
// upload only (BVH built separately so both phases are timed)
void upload(pierce_ctx* ctx, const HostDataset& h, GpuDataset& g);
void build_index(pierce_ctx* ctx, GpuDataset& g);

struct Estimate {
    int matched_cells = 0;
    double raw = 0.0;
    long long pairs = 0;
    float avg_size[2] = {0, 0}, avg_ratio[2] = {1, 1}, eff_size[2] = {0, 0}, alpha = 1.0f;
    bool has_grid = false;
};
// Grid selectivity estimate (pierce_overlap_main.cpp:376-471 and its twins).
Estimate estimate_pairs(pierce_ctx* ctx, const HostDataset& a, const HostDataset& b, float epsilon, float gamma,
                        bool alpha_correction, bool verbose_mismatch);

long long micros(double ms);
void write_pairs_csv(const std::string& path, const char* header, const std::vector<pierce_pair>& pairs);
std::vector<pierce_pair> download(pierce_ctx* ctx, pierce_result* r);
