// Unit icosphere templates, shared by the host generators and the device
// expansion (host code of instanced.cu), so both start from the same doubles.
//
// Icosahedron vertices (+-1, +-phi, 0) and their cyclic permutations are
// projected to the unit sphere; the 20 faces are oriented outward; each
// subdivision splits every triangle into four through the normalised edge
// midpoints (a shared midpoint is created once, in first-use order).  The
// unique undirected edges are listed once each, in first-seen order and
// orientation over the triangles.  Compiled with contraction of multiply-add
// disabled, so every host produces the same bits.
#pragma once

#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <utility>
#include <vector>

namespace pierce {
namespace inst {

struct IcoTemplate {
    std::vector<double> v;    // 3 per vertex, unit length
    std::vector<uint32_t> t;  // 3 per triangle, outward counter-clockwise
    std::vector<uint32_t> e;  // 2 per unique edge
};

inline void normalize3(double* p) {
    const double l = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    if (l > 0) {
        const double inv = 1.0 / l;
        p[0] *= inv;
        p[1] *= inv;
        p[2] *= inv;
    } else {
        p[0] = 0;
        p[1] = 0;
        p[2] = 1;
    }
}

inline IcoTemplate make_icosphere_template(int level) {
    IcoTemplate h;
    const double phi = (1.0 + std::sqrt(5.0)) / 2.0;
    const double raw[12][3] = {{-1, phi, 0}, {1, phi, 0},  {-1, -phi, 0}, {1, -phi, 0},
                               {0, -1, phi}, {0, 1, phi},  {0, -1, -phi}, {0, 1, -phi},
                               {phi, 0, -1}, {phi, 0, 1},  {-phi, 0, -1}, {-phi, 0, 1}};
    for (auto& r : raw) {
        double p[3] = {r[0], r[1], r[2]};
        normalize3(p);
        h.v.insert(h.v.end(), p, p + 3);
    }
    const uint32_t faces[20][3] = {{0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11},
                                   {1, 5, 9},  {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
                                   {3, 9, 4},  {3, 4, 2},  {3, 2, 6},   {3, 6, 8},  {3, 8, 9},
                                   {4, 9, 5},  {2, 4, 11}, {6, 2, 10},  {8, 6, 7},  {9, 8, 1}};
    for (auto& f : faces) h.t.insert(h.t.end(), f, f + 3);
    for (int l = 0; l < level; ++l) {
        std::map<std::pair<uint32_t, uint32_t>, uint32_t> mid;
        auto midpoint = [&](uint32_t a, uint32_t b) -> uint32_t {
            auto key = std::make_pair(std::min(a, b), std::max(a, b));
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            double p[3] = {(h.v[3 * a] + h.v[3 * b]) * 0.5, (h.v[3 * a + 1] + h.v[3 * b + 1]) * 0.5,
                           (h.v[3 * a + 2] + h.v[3 * b + 2]) * 0.5};
            normalize3(p);
            const uint32_t id = (uint32_t)(h.v.size() / 3);
            h.v.insert(h.v.end(), p, p + 3);
            mid.emplace(key, id);
            return id;
        };
        std::vector<uint32_t> nt;
        nt.reserve(h.t.size() * 4);
        for (size_t i = 0; i < h.t.size(); i += 3) {
            const uint32_t a = h.t[i], b = h.t[i + 1], c = h.t[i + 2];
            const uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            const uint32_t four[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            nt.insert(nt.end(), four, four + 12);
        }
        h.t.swap(nt);
    }
    std::map<std::pair<uint32_t, uint32_t>, int> seen;
    for (size_t i = 0; i < h.t.size(); i += 3)
        for (int k = 0; k < 3; ++k) {
            const uint32_t a = h.t[i + k], b = h.t[i + (k + 1) % 3];
            if (seen.emplace(std::make_pair(std::min(a, b), std::max(a, b)), 1).second) {
                h.e.push_back(a);
                h.e.push_back(b);
            }
        }
    return h;
}

}  // namespace inst
}  // namespace pierce
