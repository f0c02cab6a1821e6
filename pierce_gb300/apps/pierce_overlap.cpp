// pierce_overlap: overlap join with on-the-fly hash de-duplication and
// grid-estimated table sizing.  Flags, stdout lines and timing-JSON keys
// follow pierce/query/src/applications/pierce_overlap_main.cpp:221-749; the
// OptiX work is replaced by the C ABI of libpierce_gb300.
#include <cmath>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "app_common.h"
#include "cli.h"
#include "timer.h"

namespace {

const char* dir_name(int d) {
    return d == PIERCE_MESH1_TO_MESH2 ? "mesh1_to_mesh2" : (d == PIERCE_MESH2_TO_MESH1 ? "mesh2_to_mesh1" : "both");
}

struct Options : CliBase {
    Options() : CliBase("estimated_overlap_timing.json") {}
    bool estimate_only = false, track_contention = false, alpha_correction = true, valid = true;
    float gamma = 0.8f, epsilon = 0.001f, free_mem_fraction = 0.0f;
    int direction = PIERCE_BOTH, max_iterations = 100;
    std::string pairs_output;
    unsigned long long manual_slots = 0;

    bool app_option(const std::string& a, int& i, int argc, char** argv) override {
        if (a == "--gamma" && i + 1 < argc) return gamma = std::stof(argv[++i]), true;
        if (a == "--epsilon" && i + 1 < argc) return epsilon = std::stof(argv[++i]), true;
        if (a == "--query-direction" && i + 1 < argc) {
            const std::string d = argv[++i];
            if (d == "both") direction = PIERCE_BOTH;
            else if (d == "mesh1_to_mesh2") direction = PIERCE_MESH1_TO_MESH2;
            else if (d == "mesh2_to_mesh1") direction = PIERCE_MESH2_TO_MESH1;
            else {
                std::cerr << "Error: Invalid --query-direction value: " << d
                          << ". Expected one of: both, mesh1_to_mesh2, mesh2_to_mesh1" << std::endl;
                valid = false;
            }
            return true;
        }
        if (a == "--pairs-output" && i + 1 < argc) return pairs_output = argv[++i], true;
        if (a == "--track-hash-contention") return track_contention = true, true;
        if (a == "--no-alpha-correction") return alpha_correction = false, true;
        if (a == "--hash-table-size" && i + 1 < argc) return manual_slots = std::stoull(argv[++i]), true;
        if (a == "--hash-table-free-mem-fraction" && i + 1 < argc) return free_mem_fraction = std::stof(argv[++i]), true;
        if (a == "--estimate-only") return estimate_only = true, true;
        // All hits of a segment are collected in one traversal, so the
        // iteration cap of the reference's re-trace loop has no effect.
        if (a == "--overlap-max-iterations" && i + 1 < argc) return max_iterations = std::stoi(argv[++i]), true;
        return false;
    }

    void usage(const char* exe) const {
        std::vector<Entry> o;
        common_help(o);
        o.emplace_back("--gamma <float>", "Gamma parameter for estimation (default: 0.8)");
        o.emplace_back("--epsilon <float>", "Epsilon parameter for estimation (default: 0.001)");
        o.emplace_back("--query-direction <d>", "Query direction: both|mesh1_to_mesh2|mesh2_to_mesh1 (default: both)");
        o.emplace_back("--pairs-output <path>", "Optional CSV export path for unique result pairs");
        o.emplace_back("--track-hash-contention", "Track hash accesses and contention rate");
        o.emplace_back("--no-alpha-correction", "Disable replication-factor alpha correction for estimated pairs");
        o.emplace_back("--hash-table-size <ull>", "Override hash table size (slots); 0 = auto-compute");
        o.emplace_back("--hash-table-free-mem-fraction <f>", "Use f in (0,1] of free GPU memory for hash table sizing");
        o.emplace_back("--overlap-max-iterations <int>", "Accepted; every hit is collected in one traversal");
        o.emplace_back("--estimate-only", "Only run selectivity estimation, skip actual query");
        o.emplace_back("--help, -h", "Show this help message");
        print_help(exe, "--mesh1 <path> --mesh2 <path> [options]",
                   "Overlap direct-estimation query with optional pair export and hash contention diagnostics.", o);
    }
};

}  // namespace

int main(int argc, char** argv) {
    PhaseTimer timer;
    Options opt;
    opt.parse(argc, argv);
    if (opt.help) {
        opt.usage(argv[0]);
        return 0;
    }
    if (!opt.valid) return 1;
    opt.sanitize();
    if (!opt.has_meshes()) {
        std::cerr << "Usage: " << argv[0] << " --mesh1 <path> --mesh2 <path> [options]" << std::endl;
        return 1;
    }
    if (opt.free_mem_fraction < 0.0f || opt.free_mem_fraction > 1.0f) {
        std::cerr << "Error: --hash-table-free-mem-fraction must be in [0, 1]." << std::endl;
        return 1;
    }

    timer.start("Load Mesh1");
    HostDataset m1, m2;
    if (!load_dataset(opt.mesh1, m1)) {
        std::cerr << "Error loading mesh1." << std::endl;
        return 1;
    }
    if (!require_edges(m1, opt.mesh1, "Mesh1")) return 1;
    timer.next("Load Mesh2");
    if (!load_dataset(opt.mesh2, m2)) {
        std::cerr << "Error loading mesh2." << std::endl;
        return 1;
    }
    if (!require_edges(m2, opt.mesh2, "Mesh2")) return 1;

    pierce_ctx* ctx = nullptr;
    check(pierce_ctx_create(0, &ctx), "GPU context");

    auto estimate = [&]() { return estimate_pairs(ctx, m1, m2, opt.epsilon, opt.gamma, opt.alpha_correction, false); };
    // computeHashTableSize (pierce_overlap_main.cpp:473-501)
    auto table_size = [&](long long est) -> unsigned long long {
        if (opt.free_mem_fraction > 0.0f) {
            uint64_t fr = 0, tot = 0;
            if (pierce_device_memory(ctx, &fr, &tot) == PIERCE_OK && fr > 0) {
                unsigned long long slots = (unsigned long long)((double)opt.free_mem_fraction * (double)fr) / 8ull;
                if (slots < 1024ull) slots = 1024ull;
                if (slots % 2ull == 0ull) slots += 1ull;
                return slots;
            }
            std::cerr << "Warning: cudaMemGetInfo failed for free-memory hash sizing. Falling back to estimate-based "
                         "sizing." << std::endl;
        }
        unsigned long long size = 16777216ull;
        if (est > 0) {
            unsigned long long target = (unsigned long long)((double)est / 0.5);
            if (target < 1024) target = 1024;
            if (target > 2147483648ull) target = 2147483648ull;
            size = target;
            if (size % 2 == 0) size++;
        }
        return size;
    };
    auto print_sizing = [&](long long est, unsigned long long size) {
        std::cout << "\n=== Selectivity Estimation (Overlap - Direct) ===" << std::endl;
        std::cout << "Final Estimated Pairs:     " << est << std::endl;
        if (opt.manual_slots > 0) std::cout << "Using Manual Hash Table Size: " << size << std::endl;
        else if (opt.free_mem_fraction > 0.0f) std::cout << "Using Free GPU Memory Hash Table Size: " << size << std::endl;
        else std::cout << "Using Direct Estimated Hash Table Size: " << size << std::endl;
        std::cout << "Hash Table Allocated Bytes: " << size * 8ull << std::endl;
    };

    if (opt.estimate_only) {
        timer.next("Selectivity Estimation");
        const Estimate e = estimate();
        const unsigned long long size = opt.manual_slots > 0 ? opt.manual_slots : table_size(e.pairs);
        print_sizing(e.pairs, size);
        timer.finish(opt.output_json);
        pierce_ctx_destroy(ctx);
        return 0;
    }

    timer.next("Init GPU");
    timer.next("Upload Mesh1");
    GpuDataset g1, g2;
    upload(ctx, m1, g1);
    timer.next("Upload Mesh2");
    upload(ctx, m2, g2);
    timer.next("Build Mesh1 Index");
    build_index(ctx, g1);
    timer.next("Build Mesh2 Index");
    build_index(ctx, g2);
    timer.next("Upload Mesh1 Edges");
    std::cout << "Mesh1 edges uploaded: " << m1.view.num_edges << " unique edges" << std::endl;
    timer.next("Upload Mesh2 Edges");
    std::cout << "Mesh2 edges uploaded: " << m2.view.num_edges << " unique edges" << std::endl;
    timer.next("Prepare Kernel Parameters");

    auto run_query = [&](long long est, unsigned long long size, bool verbose, pierce_stats* st) {
        pierce_join_opts o;
        pierce_default_join_opts(&o);
        o.predicate = PIERCE_OVERLAP;
        o.direction = opt.direction;
        o.sizing = PIERCE_SIZING_FIXED;
        o.hash_table_slots = size;
        o.expected_pairs = est > 0 ? (uint64_t)est : 0;
        pierce_result* r = nullptr;
        check(pierce_join(ctx, g1.ds, g2.ds, &o, &r, st), "hash query");
        uint64_t n = 0;
        pierce_result_count(r, &n);
        if (verbose) std::cout << "Hash Table Query found " << n << " unique pairs." << std::endl;
        return r;
    };

    timer.next("Warmup");
    if (opt.warmup_runs > 0) {
        std::cout << "Running " << opt.warmup_runs << " warmup iterations (estimation + hash query)..." << std::endl;
        for (int w = 0; w < opt.warmup_runs; ++w) {
            const Estimate e = estimate();
            pierce_stats st;
            pierce_result_destroy(run_query(e.pairs, table_size(e.pairs), false, &st));
        }
    }

    std::vector<pierce_pair> pairs;
    pierce_stats last{};
    unsigned long long last_size = 0;
    for (int run = 0; run < opt.runs; ++run) {
        const bool verbose = run == 0;
        timer.next("Selectivity Estimation");
        const Estimate e = estimate();
        const unsigned long long size = opt.manual_slots > 0 ? opt.manual_slots : table_size(e.pairs);
        timer.next("Execute Hash Query");
        if (verbose) print_sizing(e.pairs, size);
        pierce_stats st;
        pierce_result* r = run_query(e.pairs, size, verbose, &st);
        if (opt.direction != PIERCE_MESH2_TO_MESH1)
            timer.add_measurement("Raytrace_Hash_Mesh1ToMesh2", micros(st.ms_edge_rays[0]));
        if (opt.direction != PIERCE_MESH1_TO_MESH2)
            timer.add_measurement("Raytrace_Hash_Mesh2ToMesh1", micros(st.ms_edge_rays[1]));
        timer.add_measurement("compact_hash_table_pairs", micros(st.ms_dedup));
        timer.next("Download Results");
        pairs = download(ctx, r);
        pierce_result_destroy(r);
        last = st;
        last_size = st.hash_slots;
        if (opt.track_contention) {
            const double pct = st.hash_accesses ? 100.0 * (double)st.hash_contentions / (double)st.hash_accesses : 0.0;
            std::cout << std::fixed << std::setprecision(2) << "Hash contention (run " << (run + 1)
                      << "): " << st.hash_contentions << "/" << st.hash_accesses << " accesses (" << pct << "%)"
                      << std::endl;
            std::cout.unsetf(std::ios::floatfield);
        }
    }

    timer.next("Cleanup");
    std::cout << "\n=== Mesh Overlap Join Summary ===" << std::endl;
    std::cout << "Mesh1 triangles: " << m1.view.num_triangles << std::endl;
    std::cout << "Mesh1 objects: " << m1.unique_objects << std::endl;
    std::cout << "Mesh2 triangles: " << m2.view.num_triangles << std::endl;
    std::cout << "Mesh2 objects: " << m2.unique_objects << std::endl;
    std::cout << "Query direction: " << dir_name(opt.direction) << std::endl;
    std::cout << "Hash contention tracking: " << (opt.track_contention ? "enabled" : "disabled") << std::endl;
    if (opt.track_contention) {
        const double pct = last.hash_accesses ? 100.0 * (double)last.hash_contentions / (double)last.hash_accesses : 0.0;
        std::cout << std::fixed << std::setprecision(2) << "Hash contention (last run): " << last.hash_contentions
                  << "/" << last.hash_accesses << " accesses (" << pct << "%)" << std::endl;
        std::cout.unsetf(std::ios::floatfield);
    }
    std::cout << "Unique object pairs: " << pairs.size() << std::endl;
    std::cout << "Result Buffer Capacity: " << last.result_capacity << std::endl;
    std::cout << "Result Buffer Allocated Bytes: " << last.result_capacity * 8ull << std::endl;
    std::cout << "Result Buffer Used Bytes: " << (unsigned long long)pairs.size() * 8ull << std::endl;
    std::cout << "Hash Table Slots: " << last_size << std::endl;
    std::cout << "Hash Table Allocated Bytes: " << last_size * 8ull << std::endl;
    if (!opt.pairs_output.empty()) {
        write_pairs_csv(opt.pairs_output, "object_id_mesh1,object_id_mesh2", pairs);
        std::cout << "Pair results written to: " << opt.pairs_output << std::endl;
    }
    timer.finish(opt.output_json);
    std::cout << "\nQuery completed in " << (double)timer.total_us() / 1000.0 << " ms." << std::endl;
    std::cout << "Results saved to: " << opt.output_json << std::endl;
    return 0;
}
