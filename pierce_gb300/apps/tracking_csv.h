// Parity-ray tracking tables of pierce_intersection --enable-tracking and
// the two CSVs written from them (pierce_intersection_main.cpp:425-539).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pierce_capi.h"

// Tracked targets of one direction's parity rays (kMaxPairTargetsPerSource
// slots per source object, as PairHitTrackingBuffers holds them), filled by
// pierce_parity_tracking; rays[s] = 1 when object s has triangles.
struct Tracking {
    static constexpr int kSlots = 256;
    int32_t num_sources = 0;
    std::vector<int32_t> ids;
    std::vector<uint32_t> hits, crossed, overflow, rays;
};

// Every tracked (odd-parity) target with its crossing count and whether the
// pair is in `pairs` (the join's result, (mesh1 id, mesh2 id)), then one
// summary row per source object; t12 holds mesh1's rays against mesh2, t21
// mesh2's against mesh1.  False when a file cannot be written.
bool write_tracking(const std::string& hits_path, const std::string& track_path, const Tracking& t12,
                    const Tracking& t21, const std::vector<pierce_pair>& pairs);
