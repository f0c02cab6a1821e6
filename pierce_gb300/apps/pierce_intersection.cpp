// pierce_intersection: overlap pairs plus first-vertex parity pairs in both
// directions, de-duplicated in one hash set.  Flags, stdout lines,
// timing-JSON keys and the pairs CSV follow
// pierce/query/src/applications/pierce_intersection_main.cpp:329-978.
#include <algorithm>
#include <iostream>
#include <string>
#include <vector>

#include "app_common.h"
#include "cli.h"
#include "timer.h"
#include "tracking_csv.h"

namespace {
struct Options : CliBase {
    Options() : CliBase("estimated_intersection_timing.json") {}
    std::string direction_arg = "both", pairs_output, pair_hits_output, tracking_output;
    bool estimate_only = false, tracking = false, profiling = false;
    float gamma = 0.8f, epsilon = 0.001f, load_factor = 0.5f;
    int max_iterations = 100;

    bool app_option(const std::string& a, int& i, int argc, char** argv) override {
        if (a == "--query-direction" && i + 1 < argc) return direction_arg = argv[++i], true;
        if (a == "--estimate-only") return estimate_only = true, true;
        if (a == "--enable-tracking") return tracking = true, true;
        if (a == "--enable-profiling-stats") return profiling = true, true;
        if (a == "--pairs-output" && i + 1 < argc) return pairs_output = argv[++i], true;
        if (a == "--pair-hits-output" && i + 1 < argc) return pair_hits_output = argv[++i], true;
        if (a == "--containment-tracking-output" && i + 1 < argc) return tracking_output = argv[++i], true;
        if (a == "--gamma" && i + 1 < argc) return gamma = std::stof(argv[++i]), true;
        if (a == "--epsilon" && i + 1 < argc) return epsilon = std::stof(argv[++i]), true;
        if (a == "--hash-load-factor" && i + 1 < argc) return load_factor = std::stof(argv[++i]), true;
        if (a == "--overlap-max-iterations" && i + 1 < argc) return max_iterations = std::stoi(argv[++i]), true;
        return false;
    }
    void usage(const char* exe) const {
        std::vector<Entry> o;
        common_help(o);
        o.emplace_back("--gamma <float>", "Estimation gamma (default: 0.8)");
        o.emplace_back("--epsilon <float>", "Estimation epsilon (default: 0.001)");
        o.emplace_back("--estimate-only", "Run only selectivity estimation");
        o.emplace_back("--query-direction <both|mesh1_to_mesh2|mesh2_to_mesh1>", "Control query direction (default: both)");
        o.emplace_back("--overlap-max-iterations <int>", "Accepted (must be > 0); every hit is collected in one traversal");
        o.emplace_back("--hash-load-factor <float>", "Hash load factor in (0,1] (default: 0.5)");
        o.emplace_back("--enable-tracking", "Write per-object summary CSVs of the join");
        o.emplace_back("--enable-profiling-stats", "Add device counters to the timing JSON");
        o.emplace_back("--pairs-output <path>", "Intersection pairs CSV path (default: intersection_pairs.csv)");
        o.emplace_back("--pair-hits-output <path>", "Pair hit tracking CSV path (default: intersection_pair_hits.csv)");
        o.emplace_back("--containment-tracking-output <path>",
                       "Containment tracking CSV path (default: intersection_containment_tracking.csv)");
        o.emplace_back("--help, -h", "Show this help message");
        print_help(exe, "--mesh1 <path> --mesh2 <path> [options]",
                   "Intersection join: overlapping surfaces or one object's first vertex inside the other.", o);
    }
};

// pierce_parity_tracking for one direction; objects without triangles trace
// no ray (iterations 0).  False (message on stderr) when the target's
// objects are not stored contiguously.
bool track(pierce_ctx* ctx, pierce_dataset* src, pierce_dataset* tgt, const HostDataset& src_host, Tracking& t) {
    pierce_dataset_info info;
    check(pierce_dataset_info_get(src, &info), "dataset info");
    t.num_sources = std::max(info.num_objects, 0);
    const size_t n = (size_t)t.num_sources;
    t.ids.assign(n * Tracking::kSlots, -1);
    t.hits.assign(n * Tracking::kSlots, 0);
    t.crossed.assign(n, 0);
    t.overflow.assign(n, 0);
    t.rays.assign(n, 0);
    for (uint64_t i = 0; i < src_host.view.num_mappings; ++i) {
        const int32_t o = src_host.view.tri_to_object[i];
        if (o >= 0 && (size_t)o < n) t.rays[o] = 1;
    }
    if (n == 0) return true;
    const int s = pierce_parity_tracking(ctx, src, tgt, Tracking::kSlots, t.ids.data(), t.hits.data(),
                                         t.crossed.data(), t.overflow.data());
    if (s != PIERCE_OK) {
        std::cerr << "Tracking unavailable: " << pierce_last_error() << std::endl;
        return false;
    }
    return true;
}
}  // namespace

int main(int argc, char** argv) {
    PhaseTimer timer;
    Options opt;
    opt.parse(argc, argv);
    if (opt.help) {
        opt.usage(argv[0]);
        return 0;
    }
    const std::string pairs_path = opt.pairs_output.empty() ? "intersection_pairs.csv" : opt.pairs_output;
    const std::string hits_path = opt.pair_hits_output.empty() ? "intersection_pair_hits.csv" : opt.pair_hits_output;
    const std::string track_path =
        opt.tracking_output.empty() ? "intersection_containment_tracking.csv" : opt.tracking_output;
    int direction = PIERCE_BOTH;
    if (opt.direction_arg == "mesh1_to_mesh2") direction = PIERCE_MESH1_TO_MESH2;
    else if (opt.direction_arg == "mesh2_to_mesh1") direction = PIERCE_MESH2_TO_MESH1;
    else if (opt.direction_arg != "both") {
        std::cerr << "Invalid query direction: " << opt.direction_arg << std::endl;
        std::cerr << "Valid values for --query-direction are: both, mesh1_to_mesh2, mesh2_to_mesh1" << std::endl;
        return 1;
    }
    if (opt.load_factor <= 0.0f || opt.load_factor > 1.0f) {
        std::cerr << "Invalid --hash-load-factor. Expected value in (0, 1]." << std::endl;
        return 1;
    }
    if (opt.max_iterations <= 0) {
        std::cerr << "--overlap-max-iterations must be > 0." << std::endl;
        return 1;
    }
    if (!opt.has_meshes()) {
        std::cerr << "Usage: " << argv[0] << " --mesh1 <path> --mesh2 <path> [options]" << std::endl;
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
    auto estimate = [&]() { return estimate_pairs(ctx, m1, m2, opt.epsilon, opt.gamma, true, false); };
    for (int w = 0; w < opt.warmup_runs; ++w) (void)estimate();

    timer.next("Selectivity Estimation");
    const Estimate e = estimate();
    // chooseIntersectionHashTableSize (pierce_intersection_main.cpp:313-327)
    long long table = 16777216;
    if (e.pairs > 0) {
        unsigned long long target = (unsigned long long)((double)e.pairs / opt.load_factor);
        if (target < 1024) target = 1024;
        if (target > 1073741824ull) target = 1073741824ull;
        table = (long long)target;
        if (table % 2 == 0) table += 1;
    }
    auto print_config = [&]() {
        std::cout << "\n=== Query Configuration ===" << std::endl;
        std::cout << "Estimated Pairs:    " << e.pairs << std::endl;
        std::cout << "Hash Table Size:    " << table << " (Load Factor ~" << opt.load_factor << ")" << std::endl;
        std::cout << "Query Direction:    " << opt.direction_arg << std::endl;
        std::cout << "Overlap Max Iter:   " << opt.max_iterations << std::endl;
        std::cout << "Tracking:           " << (opt.tracking ? "enabled" : "disabled") << std::endl;
        std::cout << "Profiling Stats:    " << (opt.profiling ? "enabled" : "disabled") << std::endl;
        std::cout << "===========================\n" << std::endl;
    };
    if (opt.estimate_only) {
        print_config();
        timer.finish(opt.output_json);
        return 0;
    }
    timer.next("Init GPU");
    print_config();
    timer.next("Upload Mesh1");
    GpuDataset g1, g2;
    upload(ctx, m1, g1);
    timer.next("Upload Mesh2");
    upload(ctx, m2, g2);
    timer.next("Build Mesh1 Index");
    build_index(ctx, g1);
    timer.next("Build Mesh2 Index");
    build_index(ctx, g2);
    timer.next("Prepare Kernel Parameters");

    pierce_join_opts o;
    pierce_default_join_opts(&o);
    o.predicate = PIERCE_INTERSECTION;
    o.direction = direction;
    o.sizing = PIERCE_SIZING_FIXED;
    o.hash_table_slots = (uint64_t)table;
    o.hash_load_factor = opt.load_factor;
    o.expected_pairs = e.pairs > 0 ? (uint64_t)e.pairs : 0;

    timer.next("Warmup");
    if (opt.warmup_runs > 0) {
        std::cout << "Running " << opt.warmup_runs << " warmup iterations (hash query)..." << std::endl;
        for (int w = 0; w < opt.warmup_runs; ++w) {
            pierce_result* r = nullptr;
            check(pierce_join(ctx, g1.ds, g2.ds, &o, &r, nullptr), "intersection query");
            pierce_result_destroy(r);
        }
    }
    timer.next("Query");
    std::cout << "Running Intersection Query..." << std::endl;
    pierce_result* r = nullptr;
    pierce_stats st;
    check(pierce_join(ctx, g1.ds, g2.ds, &o, &r, &st), "intersection query");
    const bool ab = direction != PIERCE_MESH2_TO_MESH1, ba = direction != PIERCE_MESH1_TO_MESH2;
    if (ab) timer.add_measurement("Raytrace_Overlap_Hash_Mesh1ToMesh2", micros(st.ms_edge_rays[0]));
    if (ba) timer.add_measurement("Raytrace_Overlap_Hash_Mesh2ToMesh1", micros(st.ms_edge_rays[1]));
    if (ab) timer.add_measurement("Raytrace_Containment_Hash_Mesh1ToMesh2", micros(st.ms_parity[0]));
    if (ba) timer.add_measurement("Raytrace_Containment_Hash_Mesh2ToMesh1", micros(st.ms_parity[1]));
    timer.add_measurement("compact_hash_table_pairs", micros(st.ms_dedup));
    uint64_t n = 0;
    pierce_result_count(r, &n);
    std::cout << "Hash Table Query found " << n << " unique pairs." << std::endl;
    std::cout << "Actual Intersection Pairs: " << n << std::endl;
    timer.add_counter("Profile_Actual_Intersection_Pairs", n);
    std::vector<pierce_pair> pairs = download(ctx, r);
    pierce_result_destroy(r);
    write_pairs_csv(pairs_path, "a_object_id,b_object_id", pairs);
    bool tracked = false;
    if (opt.tracking) {
        // both directions' parity rays, as the reference copies both
        // directions' tracking buffers whatever the query direction
        Tracking t12, t21;
        tracked = track(ctx, g1.ds, g2.ds, m1, t12) && track(ctx, g2.ds, g1.ds, m2, t21);
        if (tracked && !write_tracking(hits_path, track_path, t12, t21, pairs)) {
            std::cerr << "Failed to write the tracking CSVs " << hits_path << ", " << track_path << std::endl;
            return 1;
        }
    }
    std::cout << "Intersection pairs CSV: " << pairs_path << std::endl;
    if (tracked) {
        std::cout << "Pair hit tracking CSV: " << hits_path << std::endl;
        std::cout << "Containment tracking CSV: " << track_path << std::endl;
    }
    if (opt.profiling) {
        // Counters of MeshIntersectionProfilingStats (mesh_intersection.h:7-22,
        // pierce_intersection_main.cpp:924-948) that this design has: one
        // traversal per edge ray collects all its hits, so iterations equal
        // rays; no hit is suppressed and no candidate list overflows.
        const unsigned long long it_x1000 = st.rays ? 1000ull : 0ull, pit_x1000 = st.parity_rays ? 1000ull : 0ull;
        timer.add_counter("Profile_Overlap_Trace_Calls", st.rays);
        timer.add_counter("Profile_Overlap_Iterations_Total", st.rays);
        timer.add_counter("Profile_Overlap_Hits_Total", st.raw_hits);
        timer.add_counter("Profile_Overlap_Max_Iterations_Per_Trace", st.rays ? 1 : 0);
        timer.add_counter("Profile_Containment_Rays_Total", st.parity_rays);
        timer.add_counter("Profile_Containment_Iterations_Total", st.parity_rays);
        timer.add_counter("Profile_Containment_Max_Iterations_Per_Ray", st.parity_rays ? 1 : 0);
        timer.add_counter("Profile_Containment_Same_Hit_Suppressed", 0);
        timer.add_counter("Profile_Containment_Candidate_Overflow", 0);
        timer.add_counter("Profile_Overlap_Avg_Iterations_x1000", it_x1000);
        timer.add_counter("Profile_Containment_Avg_Iterations_x1000", pit_x1000);
        timer.add_counter("Profile_Node_Visits", st.node_visits);
        timer.add_counter("Profile_Triangle_Tests", st.tri_tests);
        timer.add_counter("Profile_Fp32_Ambiguous", st.fp32_ambiguous);
        timer.add_counter("Profile_Fp64_Ambiguous", st.fp64_ambiguous);
    }
    timer.next("Cleanup");
    timer.finish(opt.output_json);
    return 0;
}
