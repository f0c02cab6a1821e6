// pierce_preprocess: OBJ meshes -> `.pre` v4 file (vertices, triangles,
// triangle->object map, unique-edge payload, optional grid statistics).
// Flags follow pierce/preprocess/src/pierce_preprocess.cpp:171-333.
//
// OBJ reading follows the object model of ObjMeshDatasetLoader::load
// (pierce/preprocess/src/ObjMeshDatasetLoader.cpp:14-168) on top of
// tinyobjloader's shape rules: a new object starts at each `o` or `g` line
// that follows faces; faces with more than three corners are split into a
// fan (tinyobjloader triangulates by default); each object's used vertices
// are copied in first-use order (the reference's order is that of an
// unordered_set and therefore unspecified); shapes without faces are
// skipped.  Edges are extracted in the reference's map order.
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <random>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/pierce_host.h"
#include "timer.h"

namespace {

struct ObjData {
    std::vector<float> vertices;
    std::vector<uint32_t> indices;
    std::vector<int32_t> tri_to_object;
    int objects = 0, skipped = 0;
};

// Parse one face corner "v", "v/vt", "v//vn" or "v/vt/vn" -> 0-based vertex index.
bool corner_index(const std::string& tok, long nverts, long* out) {
    const size_t slash = tok.find('/');
    const std::string v = tok.substr(0, slash);
    if (v.empty()) return false;
    char* end = nullptr;
    const long i = std::strtol(v.c_str(), &end, 10);
    if (*end != '\0' || i == 0) return false;
    *out = i > 0 ? i - 1 : nverts + i;
    return *out >= 0;
}

bool read_obj(const std::string& path, ObjData& d) {
    std::ifstream in(path);
    if (!in) {
        std::cerr << "Error: File does not exist: " << path << std::endl;
        return false;
    }
    std::vector<float> all;  // every `v` line
    std::vector<std::vector<long>> shape_faces(1);  // corners, 3 per triangle, per shape
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ss(line);
        std::string tag;
        if (!(ss >> tag)) continue;
        if (tag == "v") {
            float x = 0, y = 0, z = 0;
            ss >> x >> y >> z;
            all.push_back(x);
            all.push_back(y);
            all.push_back(z);
        } else if (tag == "o" || tag == "g") {
            if (!shape_faces.back().empty()) shape_faces.emplace_back();
        } else if (tag == "f") {
            std::vector<long> c;
            std::string tok;
            const long nv = (long)(all.size() / 3);
            while (ss >> tok) {
                long idx = 0;
                if (!corner_index(tok, nv, &idx)) {
                    std::cerr << "Error loading .obj file: bad face corner '" << tok << "'" << std::endl;
                    return false;
                }
                c.push_back(idx);
            }
            for (size_t k = 1; k + 1 < c.size(); ++k) {
                shape_faces.back().push_back(c[0]);
                shape_faces.back().push_back(c[k]);
                shape_faces.back().push_back(c[k + 1]);
            }
        }
    }
    const long nv = (long)(all.size() / 3);
    for (const auto& faces : shape_faces) {
        if (faces.empty()) continue;
        std::unordered_map<long, uint32_t> local;
        const uint32_t base = (uint32_t)(d.vertices.size() / 3);
        bool ok = true;
        for (long v : faces)
            if (v >= nv) ok = false;
        if (!ok) {
            d.skipped++;
            continue;
        }
        for (long v : faces) {
            auto it = local.find(v);
            if (it == local.end()) {
                local.emplace(v, base + (uint32_t)local.size());
                d.vertices.insert(d.vertices.end(), &all[3 * v], &all[3 * v] + 3);
            }
        }
        for (size_t k = 0; k < faces.size(); k += 3) {
            for (int j = 0; j < 3; ++j) d.indices.push_back(local[faces[k + j]]);
            d.tri_to_object.push_back(d.objects);
        }
        d.objects++;
    }
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    std::string dataset, out_geometry = "geometry_data.txt", out_timing = "preprocessing_timing.json", mode = "mesh";
    bool shuffle = false, grid = false;
    float cell = 1.0f;
    long long seed = -1;
    std::cout << "Arguments received:" << std::endl;
    for (int i = 0; i < argc; ++i) std::cout << "  [" << i << "] " << argv[i] << std::endl;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--dataset" && i + 1 < argc) dataset = argv[++i];
        else if (a == "--mode" && i + 1 < argc) mode = argv[++i];
        else if (a == "--output-geometry" && i + 1 < argc) out_geometry = argv[++i];
        else if (a == "--output-timing" && i + 1 < argc) out_timing = argv[++i];
        else if (a == "--shuffle" || a == "shuffle") shuffle = true;
        else if (a == "--seed" && i + 1 < argc) seed = std::atoll(argv[++i]);
        else if (a == "--generate-grid") grid = true;
        else if (a == "--grid-cell-size" && i + 1 < argc) cell = std::stof(argv[++i]);
        else if (a == "--gamma" && i + 1 < argc) ++i;
        else if (a == "--help" || a == "-h") {
            std::cout << "Usage: " << argv[0]
                      << " [--mode <mesh|dt>] [--dataset <path>] [--output-geometry <geometry_output_file>] "
                         "[--output-timing <timing_output_file>]\n"
                         "Options:\n"
                         "  --mode <mesh|dt>           Dataset loading mode (default: mesh; dt is not supported)\n"
                         "  --dataset <path>           Path to dataset (.obj)\n"
                         "  --output-geometry <path>   Path of the .pre output\n"
                         "  --output-timing <path>     Path to JSON file for preprocessing timing output\n"
                         "  --shuffle                  Randomly translate each loaded object (within +-15)\n"
                         "  --seed <n>                 Seed for --shuffle (default: random device)\n"
                         "  --generate-grid            Generate grid statistics for selectivity estimation\n"
                         "  --grid-cell-size <S>       Grid cell size (default: 1.0)"
                      << std::endl;
            return 0;
        } else {
            std::cout << "Warning: Unknown argument '" << a << "'" << std::endl;
        }
    }
    if (mode != "mesh" && mode != "dt") {
        std::cerr << "Error: Unknown mode '" << mode << "'. Valid modes: mesh, dt" << std::endl;
        return 1;
    }
    if (mode == "dt") {
        std::cerr << "Error: .dt (TDBase) datasets are not supported by this build; convert them to .obj" << std::endl;
        return 1;
    }
    if (dataset.empty()) {
        std::cerr << "Error: Dataset path is required. Use --dataset <path>" << std::endl;
        return 1;
    }
    std::cout << "Dataset Preprocessing Tool" << std::endl;
    std::cout << "Mode: " << mode << std::endl;
    std::cout << "Input dataset: " << dataset << std::endl;
    std::cout << "Output geometry: " << out_geometry << std::endl;
    std::cout << "Output timing: " << out_timing << std::endl;

    PhaseTimer timer;
    timer.start("Loading Dataset");
    if (dataset.size() < 4 || dataset.substr(dataset.size() - 4) != ".obj") {
        std::cerr << "Error: Unsupported dataset format: " << dataset << std::endl;
        return 1;
    }
    ObjData d;
    if (!read_obj(dataset, d) || d.vertices.empty()) {
        std::cerr << "Error: Failed to load dataset or dataset is empty." << std::endl;
        return 1;
    }
    std::cout << "Successfully loaded " << d.objects << " object(s)" << std::endl;
    std::cout << "Skipped " << d.skipped << " object(s)" << std::endl;
    std::cout << "Total vertices: " << d.vertices.size() / 3 << std::endl;
    std::cout << "Total triangles: " << d.tri_to_object.size() << std::endl;

    if (shuffle) {
        timer.next("Shuffling Objects (Random Translation)");
        std::mt19937 rng(seed >= 0 ? (uint32_t)seed : std::random_device{}());
        std::uniform_real_distribution<float> dist(-15.0f, 15.0f);
        std::vector<std::vector<uint32_t>> verts_of(d.objects);
        std::vector<int32_t> owner(d.vertices.size() / 3, -1);
        for (size_t t = 0; t < d.tri_to_object.size(); ++t)
            for (int j = 0; j < 3; ++j) owner[d.indices[3 * t + j]] = d.tri_to_object[t];
        for (size_t v = 0; v < owner.size(); ++v)
            if (owner[v] >= 0) verts_of[owner[v]].push_back((uint32_t)v);
        std::cout << "Applying random translations to " << d.objects << " objects..." << std::endl;
        for (int o = 0; o < d.objects; ++o) {
            const float tx = dist(rng), ty = dist(rng), tz = dist(rng);
            for (uint32_t v : verts_of[o]) {
                d.vertices[3 * v] += tx;
                d.vertices[3 * v + 1] += ty;
                d.vertices[3 * v + 2] += tz;
            }
        }
    }
    pierce_geom* g = nullptr;
    if (pierce_geom_create(d.vertices.data(), d.vertices.size() / 3, d.indices.data(), d.tri_to_object.size(),
                           d.tri_to_object.data(), &g) != PIERCE_HOST_OK) {
        std::cerr << "Error: " << pierce_host_last_error() << std::endl;
        return 1;
    }
    if (grid) {
        timer.next("Generating Grid Statistics");
        pierce_geom_grid_stats(g, cell);
        pierce_geom_view v;
        pierce_geom_get_view(g, &v);
        std::cout << "Grid statistics generated. Cell Size: " << cell << ". Populated sparse cells: "
                  << v.num_grid_cells << std::endl;
    }
    timer.next("Extracting Edges");
    pierce_geom_extract_edges(g, 0, 0);
    pierce_geom_view v;
    pierce_geom_get_view(g, &v);
    if (!v.has_edges) {
        std::cerr << "Error: Edge extraction failed. No valid edge payload generated." << std::endl;
        return 1;
    }
    std::cout << "Extracted " << v.num_edges << " unique edges (per object)" << std::endl;
    timer.next("Writing Geometry Data");
    if (pierce_geom_write_pre(g, out_geometry.c_str()) != PIERCE_HOST_OK) {
        std::cerr << "Error: " << pierce_host_last_error() << std::endl;
        return 1;
    }
    std::cout << "Geometry data written to: " << out_geometry << " (Binary)" << std::endl;
    timer.finish(out_timing);
    std::cout << "Total objects (triangles): " << v.total_triangles << std::endl;
    pierce_geom_free(g);
    return 0;
}
