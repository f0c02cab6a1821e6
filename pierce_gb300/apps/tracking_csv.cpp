// CSV output of the parity-ray tracking tables (pierce_intersection
// --enable-tracking), formats of pierce_intersection_main.cpp:425-539.
#include "tracking_csv.h"

#include <fstream>
#include <unordered_set>

namespace {
inline unsigned long long pair_key(int32_t a, int32_t b) {
    return ((unsigned long long)(uint32_t)a << 32) | (uint32_t)b;
}

}  // namespace

// Crossing counts follow the exact parity rule (each triangle the ray
// crosses under the symbolic perturbation counts once); candidate_count is
// the number of target objects the ray crosses (no list cap),
// candidate_overflow_events the odd targets beyond the 256 slots.
bool write_tracking(const std::string& hits_path, const std::string& track_path, const Tracking& t12,
                    const Tracking& t21, const std::vector<pierce_pair>& pairs) {
    std::unordered_set<unsigned long long> final_pairs;
    final_pairs.reserve(2 * pairs.size() + 1);
    for (const auto& p : pairs) final_pairs.insert(pair_key(p.a, p.b));
    const Tracking* dirs[2] = {&t12, &t21};
    const char* names[2] = {"mesh1_to_mesh2", "mesh2_to_mesh1"};
    auto is_final = [&](int d, int32_t src, int32_t tgt) {
        return final_pairs.count(d == 0 ? pair_key(src, tgt) : pair_key(tgt, src)) > 0;
    };
    std::ofstream h(hits_path);
    if (!h) return false;
    h << "direction,source_object_id,target_object_id,target_ray_hits,final_pair\n";
    for (int d = 0; d < 2; ++d) {
        const Tracking& t = *dirs[d];
        for (int32_t s = 0; s < t.num_sources; ++s)
            for (int i = 0; i < Tracking::kSlots; ++i) {
                const size_t at = (size_t)s * Tracking::kSlots + i;
                if (t.ids[at] < 0) continue;
                h << names[d] << ',' << s << ',' << t.ids[at] << ',' << t.hits[at] << ','
                  << (is_final(d, s, t.ids[at]) ? 1 : 0) << "\n";
            }
    }
    std::ofstream c(track_path);
    if (!c) return false;
    c << "direction,source_object_id,iterations,candidate_count,tracked_target_count,tracked_hit_total,"
         "candidate_overflow_events,final_pair_count,tracked_final_pair_count\n";
    for (int d = 0; d < 2; ++d) {
        const Tracking& t = *dirs[d];
        for (int32_t s = 0; s < t.num_sources; ++s) {
            int tracked = 0, tracked_final = 0;
            unsigned long long hit_total = 0;
            for (int i = 0; i < Tracking::kSlots; ++i) {
                const size_t at = (size_t)s * Tracking::kSlots + i;
                if (t.ids[at] < 0) continue;
                ++tracked;
                hit_total += t.hits[at];
                if (is_final(d, s, t.ids[at])) ++tracked_final;
            }
            c << names[d] << ',' << s << ',' << t.rays[s] << ',' << t.crossed[s] << ',' << tracked << ','
              << hit_total << ',' << t.overflow[s] << ',' << tracked_final << ',' << tracked_final << "\n";
        }
    }
    return bool(h) && bool(c);
}
