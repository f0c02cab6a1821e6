// pierce_overlap_two_pass: overlap join sized exactly by counting first
// (count, scan, write, sort + unique).  Flags, stdout lines, timing-JSON keys
// and the CSV follow
// pierce/query/src/applications/pierce_overlap_two_pass_main.cpp:39-396.
#include <algorithm>
#include <iostream>
#include <string>
#include <vector>

#include "app_common.h"
#include "cli.h"
#include "timer.h"

namespace {
struct Options : CliBase {
    Options() : CliBase("mesh_overlap_timing.json") { allow_no_export = true; }
    void usage(const char* exe) const {
        std::vector<Entry> o;
        common_help(o);
        o.emplace_back("--no-export", "Do not export results to CSV");
        o.emplace_back("--help, -h", "Show this help message");
        print_help(exe,
                   "[--mesh1 <path>] [--mesh2 <path>] [--output <json_output_file>] [--runs <number>] [--ptx <ptx_file>]",
                   "Mesh overlap join query for reporting overlapping object pairs between two datasets.", o);
    }
};
}  // namespace

int main(int argc, char** argv) {
    PhaseTimer timer;
    timer.start("Data Reading");
    Options opt;
    opt.parse(argc, argv);
    if (opt.help) {
        opt.usage(argv[0]);
        return 0;
    }
    opt.sanitize();
    std::cout << "Mesh-to-Mesh Overlap Join" << std::endl;
    if (opt.mesh1.empty()) {
        std::cerr << "Error: Mesh1 file path is required. Use --mesh1 <path_to_mesh1_file>" << std::endl;
        return 1;
    }
    if (opt.mesh2.empty()) {
        std::cerr << "Error: Mesh2 file path is required. Use --mesh2 <path_to_mesh2_file>" << std::endl;
        return 1;
    }
    timer.next("Application Creation");
    pierce_ctx* ctx = nullptr;
    check(pierce_ctx_create(0, &ctx), "GPU context");

    HostDataset m1, m2;
    timer.next("Load Mesh1");
    std::cout << "Loading Mesh1 from: " << opt.mesh1 << std::endl;
    if (!load_dataset(opt.mesh1, m1)) {
        std::cerr << "Error: Failed to load Mesh1 from " << opt.mesh1 << std::endl;
        return 1;
    }
    if (!require_edges(m1, opt.mesh1, "Mesh1")) return 1;
    std::cout << "Mesh1 loaded: " << m1.view.num_vertices << " vertices, " << m1.view.num_triangles << " triangles"
              << std::endl;
    timer.next("Load Mesh2");
    std::cout << "Loading Mesh2 from: " << opt.mesh2 << std::endl;
    if (!load_dataset(opt.mesh2, m2)) {
        std::cerr << "Error: Failed to load Mesh2 from " << opt.mesh2 << std::endl;
        return 1;
    }
    if (!require_edges(m2, opt.mesh2, "Mesh2")) return 1;
    std::cout << "Mesh2 loaded: " << m2.view.num_vertices << " vertices, " << m2.view.num_triangles << " triangles"
              << std::endl;

    GpuDataset g1, g2;
    timer.next("Upload Mesh1");
    upload(ctx, m1, g1);
    std::cout << "Mesh1 uploaded to GPU" << std::endl;
    timer.next("Upload Mesh2");
    upload(ctx, m2, g2);
    std::cout << "Mesh2 uploaded to GPU" << std::endl;
    timer.next("Build Mesh1 Index");
    build_index(ctx, g1);
    std::cout << "Mesh1 acceleration structure built" << std::endl;
    timer.next("Build Mesh2 Index");
    build_index(ctx, g2);
    std::cout << "Mesh2 acceleration structure built" << std::endl;
    timer.next("Upload Mesh1");
    std::cout << "Mesh1 edges uploaded: " << m1.view.num_edges << " unique edges" << std::endl;
    timer.next("Upload Mesh2");
    std::cout << "Mesh2 edges uploaded: " << m2.view.num_edges << " unique edges" << std::endl;
    timer.next("Create Launcher");
    timer.next("Prepare Kernel Parameters");

    pierce_join_opts o;
    pierce_default_join_opts(&o);
    o.predicate = PIERCE_OVERLAP;
    o.sizing = PIERCE_SIZING_TWO_PASS;

    timer.next("Warmup");
    if (opt.warmup_runs > 0) {
        std::cout << "Running " << opt.warmup_runs << " warmup iterations (edge-optimized)..." << std::endl;
        for (int w = 0; w < opt.warmup_runs; ++w) {
            pierce_result* r = nullptr;
            check(pierce_join(ctx, g1.ds, g2.ds, &o, &r, nullptr), "two-pass query");
            pierce_result_destroy(r);
        }
    }

    timer.next("Query");
    std::cout << "\n=== Executing mesh overlap detection (edge-optimized) ===" << std::endl;
    pierce_result* r = nullptr;
    pierce_stats st;
    check(pierce_join(ctx, g1.ds, g2.ds, &o, &r, &st), "two-pass query");
    timer.add_measurement("Raytrace_Mesh1ToMesh2_Pass1", micros(st.ms_count_pass[0]));
    timer.add_measurement("Raytrace_Mesh2ToMesh1_Pass1", micros(st.ms_count_pass[1]));
    std::cout << "Pass 1 (Optimized): Found " << st.raw_pairs[0] << " (edges) + " << st.raw_pairs[1]
              << " (edges mesh2->mesh1) = " << (st.raw_pairs[0] + st.raw_pairs[1]) << " potential overlaps."
              << std::endl;
    timer.add_measurement("Raytrace_Mesh1ToMesh2_Pass2", micros(st.ms_edge_rays[0] - st.ms_count_pass[0]));
    timer.add_measurement("Raytrace_Mesh2ToMesh1_Pass2", micros(st.ms_edge_rays[1] - st.ms_count_pass[1]));
    timer.add_measurement("gpu deduplication", micros(st.ms_dedup));
    uint64_t n = 0;
    pierce_result_count(r, &n);
    std::cout << "Deduplication: Found " << n << " unique object pairs." << std::endl;

    timer.next("Download Results");
    std::vector<pierce_pair> pairs = download(ctx, r);
    pierce_result_destroy(r);

    timer.next("Output");
    const unsigned long long raw = st.raw_pairs[0] + st.raw_pairs[1];
    std::cout << "\n=== Mesh Overlap Join Summary ===" << std::endl;
    std::cout << "Mesh1 triangles: " << m1.view.num_triangles << std::endl;
    std::cout << "Mesh1 objects: " << m1.unique_objects << std::endl;
    std::cout << "Mesh2 triangles: " << m2.view.num_triangles << std::endl;
    std::cout << "Mesh2 objects: " << m2.unique_objects << std::endl;
    std::cout << "Unique object pairs: " << n << std::endl;
    std::cout << "Result Buffer Capacity: " << raw << std::endl;
    std::cout << "Result Buffer Allocated Bytes: " << raw * 8ull << std::endl;
    std::cout << "Result Buffer Used Bytes: " << n * 8ull << std::endl;
    if (opt.export_results) {
        // The reference's order: its sort runs on the 8-byte record read as a
        // little-endian integer, i.e. by (mesh2 id, mesh1 id).
        std::stable_sort(pairs.begin(), pairs.end(), [](const pierce_pair& x, const pierce_pair& y) {
            return (uint32_t)x.b != (uint32_t)y.b ? (uint32_t)x.b < (uint32_t)y.b : (uint32_t)x.a < (uint32_t)y.a;
        });
        std::cout << "Exporting results to mesh_overlap_results.csv" << std::endl;
        write_pairs_csv("mesh_overlap_results.csv", "object_id_mesh1,object_id_mesh2", pairs);
    }
    timer.next("Cleanup");
    timer.finish(opt.output_json);
    return 0;
}
