// pierce_containment: pairs (A, B) where B's first vertex lies inside A by
// ray parity and the surfaces do not meet.  Flags, stdout lines, timing-JSON
// keys and the CSV follow
// pierce/query/src/applications/pierce_containment_main.cpp:171-644.
#include <chrono>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "app_common.h"
#include "cli.h"
#include "timer.h"

namespace {
struct Options : CliBase {
    Options() : CliBase("containment_timing.json") { allow_no_export = true; }
    bool include_overlap = false;
    int max_iterations = 256;
    float gamma = 0.8f, epsilon = 0.001f, load_factor = 0.5f;
    bool app_option(const std::string& a, int& i, int argc, char** argv) override {
        if (a == "--include-overlap-pairs") return include_overlap = true, true;
        if (a == "--overlap-max-iterations" && i + 1 < argc) return max_iterations = std::stoi(argv[++i]), true;
        if (a == "--gamma" && i + 1 < argc) return gamma = std::stof(argv[++i]), true;
        if (a == "--epsilon" && i + 1 < argc) return epsilon = std::stof(argv[++i]), true;
        if (a == "--hash-load-factor" && i + 1 < argc) return load_factor = std::stof(argv[++i]), true;
        return false;
    }
    void usage(const char* exe) const {
        std::vector<Entry> o;
        common_help(o, "Dataset A (container meshes)", "Dataset B (objects tested for containment)");
        o.emplace_back("--include-overlap-pairs",
                       "Include overlap/touch pairs in output (union of overlap + strict containment)");
        o.emplace_back("--overlap-max-iterations <int>", "Accepted; every hit is collected in one traversal");
        o.emplace_back("--gamma <float>", "Estimation gamma (default: 0.8)");
        o.emplace_back("--epsilon <float>", "Estimation epsilon (default: 0.001)");
        o.emplace_back("--hash-load-factor <float>", "Hash load factor for table sizing (default: 0.5)");
        o.emplace_back("--no-export", "Do not export results to CSV");
        o.emplace_back("--help, -h", "Show this help message");
        print_help(exe, "--mesh1 <A_dataset> --mesh2 <B_dataset> [options]",
                   "Containment query: finds pairs where B objects are fully contained in A objects.", o);
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
    std::cout << "=== Mesh Containment Query ===" << std::endl;
    std::cout << "(checks which B-objects are fully contained inside A-objects)" << std::endl;
    std::cout << "Point-in-mesh mode: exact parity" << std::endl;
    std::cout << "Include overlap pairs: " << (opt.include_overlap ? "yes" : "no") << std::endl;
    if (!opt.has_meshes()) {
        if (opt.mesh1.empty()) std::cerr << "Error: --mesh1 (dataset A) required\n";
        if (opt.mesh2.empty()) std::cerr << "Error: --mesh2 (dataset B) required\n";
        return 1;
    }
    timer.next("Application Creation");
    pierce_ctx* ctx = nullptr;
    check(pierce_ctx_create(0, &ctx), "GPU context");

    HostDataset a, b;
    timer.next("Load Mesh A");
    std::cout << "Loading dataset A from: " << opt.mesh1 << std::endl;
    if (!load_dataset(opt.mesh1, a)) {
        std::cerr << "Failed to load A\n";
        return 1;
    }
    if (!require_edges(a, opt.mesh1, "MeshA")) return 1;
    std::cout << "  A: " << a.view.num_vertices << " vertices, " << a.view.num_triangles << " triangles" << std::endl;
    timer.next("Load Mesh B");
    std::cout << "Loading dataset B from: " << opt.mesh2 << std::endl;
    if (!load_dataset(opt.mesh2, b)) {
        std::cerr << "Failed to load B\n";
        return 1;
    }
    if (!require_edges(b, opt.mesh2, "MeshB")) return 1;
    std::cout << "  B: " << b.view.num_vertices << " vertices, " << b.view.num_triangles << " triangles" << std::endl;
    std::cout << "  A objects: " << a.unique_objects << "   B objects: " << b.unique_objects << std::endl;

    GpuDataset ga, gb;
    timer.next("Upload Mesh A");
    upload(ctx, a, ga);
    timer.next("Upload Mesh B");
    upload(ctx, b, gb);
    timer.next("Build A Index");
    build_index(ctx, ga);
    timer.next("Build B Index");
    build_index(ctx, gb);
    timer.next("Prepare Kernel Parameters");

    // chooseContainmentHashTableSize (pierce_containment_main.cpp:138-150)
    auto table_size = [&](long long est) -> long long {
        if (est <= 0) return 16777216;
        unsigned long long t = (unsigned long long)((double)est / opt.load_factor);
        if (t < 1024) t = 1024;
        if (t > 536870912ull) t = 536870912ull;
        long long s = (long long)t;
        if (s % 2 == 0) s++;
        return s;
    };
    struct RunResult {
        std::vector<pierce_pair> pairs;
        uint64_t containment = 0, overlap = 0;
    };
    auto run_once = [&](bool verbose, bool record) {
        const Estimate e = estimate_pairs(ctx, a, b, opt.epsilon, opt.gamma, true, false);
        const long long size = table_size(e.pairs);
        if (verbose) {
            std::cout << "\n=== Containment Selectivity Estimation ===" << std::endl;
            std::cout << "Final Estimated Pairs:     " << e.pairs << std::endl;
            std::cout << "Hash Table Size:           " << size << " (Load Factor ~" << opt.load_factor << ")"
                      << std::endl;
            std::cout << "==========================================\n" << std::endl;
        }
        pierce_join_opts o;
        pierce_default_join_opts(&o);
        o.predicate = PIERCE_CONTAINMENT;
        o.sizing = PIERCE_SIZING_FIXED;
        o.hash_table_slots = (uint64_t)size;
        o.hash_load_factor = opt.load_factor;
        o.expected_pairs = e.pairs > 0 ? (uint64_t)e.pairs : 0;
        o.include_overlap_pairs = opt.include_overlap ? 1 : 0;
        pierce_result* r = nullptr;
        pierce_stats st;
        auto t0 = std::chrono::high_resolution_clock::now();
        check(pierce_join(ctx, ga.ds, gb.ds, &o, &r, &st), "containment query");
        (void)t0;
        RunResult rr;
        rr.containment = st.containment_pairs;
        rr.overlap = st.overlap_pairs;
        if (record) {
            timer.add_measurement("Raytrace_Overlap_Hash_Mesh2ToMesh1", micros(st.ms_edge_rays[1]));
            timer.add_measurement("Raytrace_Overlap_Hash_Mesh1ToMesh2", micros(st.ms_edge_rays[0]));
            timer.add_measurement("Raytrace_Containment_Hash_Mesh2ToMesh1", micros(st.ms_parity[1]));
            timer.add_measurement("compact_hash_table_pairs (containment)", micros(st.ms_dedup));
        }
        if (verbose) {
            std::cout << "Containment pairs found: " << rr.containment << std::endl;
            if (opt.include_overlap) std::cout << "Overlap/touch pairs found: " << rr.overlap << std::endl;
        }
        rr.pairs = download(ctx, r);
        pierce_result_destroy(r);
        return rr;
    };

    timer.next("Warmup");
    if (opt.warmup_runs > 0) {
        std::cout << "Running " << opt.warmup_runs << " warmup iterations..." << std::endl;
        for (int w = 0; w < opt.warmup_runs; ++w) run_once(false, false);
    }
    timer.next("Query");
    std::cout << "\n=== Executing containment query ===" << std::endl;
    RunResult fin;
    for (int run = 0; run < opt.runs; ++run) fin = run_once(run == opt.runs - 1, true);
    timer.next("Download Results");
    timer.next("Output");
    std::cout << "\n=== Containment Query Summary ===" << std::endl;
    std::cout << "A triangles: " << a.view.num_triangles << "  objects: " << a.unique_objects << std::endl;
    std::cout << "B triangles: " << b.view.num_triangles << "  objects: " << b.unique_objects << std::endl;
    std::cout << "Containment pairs (B in A): " << fin.containment << std::endl;
    if (opt.include_overlap) {
        std::cout << "Overlap/Touch pairs (A vs B): " << fin.overlap << std::endl;
        std::cout << "Reported pairs: " << fin.pairs.size() << std::endl;
    }
    if (opt.export_results) {
        const std::string csv = "mesh_containment_results.csv";
        std::cout << "Exporting results to " << csv << std::endl;
        std::ofstream f(csv);
        if (opt.include_overlap) {
            f << "a_object_id,b_object_id,pair_type\n";
            for (size_t i = 0; i < fin.pairs.size(); ++i)
                f << fin.pairs[i].a << "," << fin.pairs[i].b << "," << (i < fin.containment ? "containment" : "overlap")
                  << "\n";
        } else {
            f << "a_object_id,b_object_id\n";
            for (const auto& p : fin.pairs) f << p.a << "," << p.b << "\n";
        }
    }
    timer.next("Cleanup");
    timer.finish(opt.output_json);
    std::cout << "\nContainment query completed successfully." << std::endl;
    return 0;
}
