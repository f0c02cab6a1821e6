// `.pre` version-4 reader and writer.
//
// File layout (little-endian, native struct packing), as defined by
// RaySpace::IO::FileHeader and readBinaryFile/writeBinaryFile in
// pierce/common/include/BinaryIO.h:11-151:
//   56-byte header: u32 magic 0x52334442, u32 version 4, u64 numVertices,
//     u64 numIndices (triangles), u64 numMappings, u64 numEdges,
//     u64 totalTriangles, u8 hasGrid, u8 hasEdges, u8 padding[6]
//   float3 vertices[numVertices]; uint3 indices[numIndices];
//   int32 triangleToObject[numMappings];
//   if hasEdges: float3 starts[numEdges], float3 ends[numEdges], int32 src[numEdges]
//   if hasGrid: {f32 cellSize; u32 numSparseCells} + 28-byte cells
// The reader differs from the reference only in that short reads are reported
// as errors instead of leaving zero-filled arrays; a wrong magic or version is
// an error in both (BinaryIO.h:95-108).
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

#include "geometry.h"

namespace {

constexpr uint32_t kMagic = 0x52334442u;
constexpr uint32_t kVersion = 4u;

#pragma pack(push, 1)
struct Header {
    uint32_t magic;
    uint32_t version;
    uint64_t num_vertices;
    uint64_t num_indices;
    uint64_t num_mappings;
    uint64_t num_edges;
    uint64_t total_triangles;
    uint8_t has_grid;
    uint8_t has_edges;
    uint8_t padding[6];
};
struct GridParams {
    float cell_size;
    uint32_t num_cells;
};
#pragma pack(pop)
static_assert(sizeof(Header) == 56, "header must be 56 bytes");
static_assert(sizeof(pierce_grid_entry) == 28, "grid entry must be 28 bytes");

struct FileCloser {
    void operator()(FILE* f) const {
        if (f) fclose(f);
    }
};
using FilePtr = std::unique_ptr<FILE, FileCloser>;

bool read_exact(FILE* f, void* dst, size_t bytes) {
    if (bytes == 0) return true;
    return fread(dst, 1, bytes, f) == bytes;
}

bool write_exact(FILE* f, const void* src, size_t bytes) {
    if (bytes == 0) return true;
    return fwrite(src, 1, bytes, f) == bytes;
}

}  // namespace

extern "C" int pierce_geom_read_pre(const char* path, pierce_geom** out) {
    if (!path || !out) {
        pierce::set_last_error("read_pre: null argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    *out = nullptr;
    FilePtr f(fopen(path, "rb"));
    if (!f) {
        pierce::set_last_error(std::string("Could not open file for reading: ") + path);
        return PIERCE_HOST_ERR_IO;
    }
    Header h;
    if (!read_exact(f.get(), &h, sizeof(h))) {
        pierce::set_last_error(std::string("Short read of header: ") + path);
        return PIERCE_HOST_ERR_IO;
    }
    if (h.magic != kMagic) {
        pierce::set_last_error(std::string("Invalid file format (Magic mismatch). File: ") + path);
        return PIERCE_HOST_ERR_MAGIC;
    }
    if (h.version != kVersion) {
        pierce::set_last_error("Unsupported binary geometry version " + std::to_string(h.version) +
                               " in file: " + path + ". Expected version 4. Re-run preprocessing.");
        return PIERCE_HOST_ERR_VERSION;
    }
    // Refuse absurd counts before allocating (corrupt headers).
    const uint64_t kMaxCount = 1ULL << 40;
    if (h.num_vertices > kMaxCount || h.num_indices > kMaxCount || h.num_mappings > kMaxCount ||
        h.num_edges > kMaxCount) {
        pierce::set_last_error(std::string("Corrupt header counts in: ") + path);
        return PIERCE_HOST_ERR_IO;
    }
    std::unique_ptr<pierce_geom> g(new pierce_geom());
    try {
        g->total_triangles = h.total_triangles;
        g->vertices.resize(3 * h.num_vertices);
        g->indices.resize(3 * h.num_indices);
        g->tri_to_object.resize(h.num_mappings);
        bool ok = read_exact(f.get(), g->vertices.data(), g->vertices.size() * sizeof(float)) &&
                  read_exact(f.get(), g->indices.data(), g->indices.size() * sizeof(uint32_t)) &&
                  read_exact(f.get(), g->tri_to_object.data(), g->tri_to_object.size() * sizeof(int32_t));
        if (ok && h.has_edges) {
            g->edge_starts.resize(3 * h.num_edges);
            g->edge_ends.resize(3 * h.num_edges);
            g->edge_src.resize(h.num_edges);
            ok = read_exact(f.get(), g->edge_starts.data(), g->edge_starts.size() * sizeof(float)) &&
                 read_exact(f.get(), g->edge_ends.data(), g->edge_ends.size() * sizeof(float)) &&
                 read_exact(f.get(), g->edge_src.data(), g->edge_src.size() * sizeof(int32_t));
        }
        if (ok && h.has_grid) {
            GridParams gp;
            ok = read_exact(f.get(), &gp, sizeof(gp));
            if (ok) {
                g->has_grid = true;
                g->grid_cell_size = gp.cell_size;
                g->grid_cells.resize(gp.num_cells);
                ok = read_exact(f.get(), g->grid_cells.data(), g->grid_cells.size() * sizeof(pierce_grid_entry));
            }
        }
        if (!ok) {
            pierce::set_last_error(std::string("Short read (truncated file): ") + path);
            return PIERCE_HOST_ERR_IO;
        }
    } catch (const std::bad_alloc&) {
        pierce::set_last_error(std::string("Out of host memory reading: ") + path);
        return PIERCE_HOST_ERR_IO;
    }
    *out = g.release();
    return PIERCE_HOST_OK;
}

extern "C" int pierce_geom_write_pre(const pierce_geom* g, const char* path) {
    if (!g || !path) {
        pierce::set_last_error("write_pre: null argument");
        return PIERCE_HOST_ERR_INVALID;
    }
    FilePtr f(fopen(path, "wb"));
    if (!f) {
        pierce::set_last_error(std::string("Could not open file for writing: ") + path);
        return PIERCE_HOST_ERR_IO;
    }
    Header h;
    std::memset(&h, 0, sizeof(h));
    h.magic = kMagic;
    h.version = kVersion;
    h.num_vertices = g->num_vertices();
    h.num_indices = g->num_triangles();
    h.num_mappings = g->tri_to_object.size();
    h.num_edges = g->edge_src.size();
    h.total_triangles = g->total_triangles;
    h.has_grid = g->has_grid ? 1 : 0;
    h.has_edges = g->has_edges() ? 1 : 0;
    bool ok = write_exact(f.get(), &h, sizeof(h)) &&
              write_exact(f.get(), g->vertices.data(), g->vertices.size() * sizeof(float)) &&
              write_exact(f.get(), g->indices.data(), g->indices.size() * sizeof(uint32_t)) &&
              write_exact(f.get(), g->tri_to_object.data(), g->tri_to_object.size() * sizeof(int32_t));
    if (ok && h.has_edges) {
        ok = write_exact(f.get(), g->edge_starts.data(), g->edge_starts.size() * sizeof(float)) &&
             write_exact(f.get(), g->edge_ends.data(), g->edge_ends.size() * sizeof(float)) &&
             write_exact(f.get(), g->edge_src.data(), g->edge_src.size() * sizeof(int32_t));
    }
    if (ok && h.has_grid) {
        GridParams gp{g->grid_cell_size, (uint32_t)g->grid_cells.size()};
        ok = write_exact(f.get(), &gp, sizeof(gp)) &&
             write_exact(f.get(), g->grid_cells.data(), g->grid_cells.size() * sizeof(pierce_grid_entry));
    }
    if (!ok) {
        pierce::set_last_error(std::string("Write failed: ") + path);
        return PIERCE_HOST_ERR_IO;
    }
    return PIERCE_HOST_OK;
}
