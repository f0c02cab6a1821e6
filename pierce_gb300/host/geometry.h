// Host-side geometry container shared by the `.pre` reader/writer, the edge
// extractor, the generators and the command-line applications.
//
// Field meanings follow GeometryData (pierce/common/include/Geometry.h:42-51):
// flat xyz vertex array, three vertex indices per triangle, one object id per
// triangle, the unique-edge payload (start, end, source object) and the
// sparse grid statistics.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pierce_host.h"

struct pierce_geom {
    std::vector<float> vertices;       // 3 * nv
    std::vector<uint32_t> indices;     // 3 * nt
    std::vector<int32_t> tri_to_object;
    uint64_t total_triangles = 0;

    std::vector<float> edge_starts;    // 3 * ne
    std::vector<float> edge_ends;      // 3 * ne
    std::vector<int32_t> edge_src;

    bool has_grid = false;
    float grid_cell_size = 0.0f;
    std::vector<pierce_grid_entry> grid_cells;

    uint64_t num_vertices() const { return vertices.size() / 3; }
    uint64_t num_triangles() const { return indices.size() / 3; }
    uint64_t num_edges() const { return edge_src.size(); }
    // The reference treats a geometry as carrying edges when the three edge
    // arrays are non-empty and of equal length (Geometry.h:28-32).
    bool has_edges() const {
        return !edge_src.empty() && edge_starts.size() == 3 * edge_src.size() &&
               edge_ends.size() == 3 * edge_src.size();
    }
    int32_t num_objects() const {
        int32_t m = -1;
        for (int32_t o : tri_to_object) m = o > m ? o : m;
        return m + 1;
    }
};

namespace pierce {
void set_last_error(const std::string& msg);

// Edge extraction used by the C entry point and by the generators.
void extract_edges(pierce_geom& g, int order, int num_threads);
// Grid statistics.
void grid_stats(pierce_geom& g, float cell_size);
}  // namespace pierce
