// Deterministic scalar math for the dataset generators.
//
// The generators must produce bit-identical float32 geometry on every host
// (x86-64 here, aarch64 on the GPU hosts), so they may not depend on the
// platform libm, whose last-ulp results differ between implementations.
// Everything below uses only IEEE-754 basic operations (+ - * / sqrt, which
// are correctly rounded) plus frexp/ldexp (exact), and the files that
// include it are compiled with -ffp-contract=off so no FMA is formed.
//
// exp and log use textbook series (Taylor for exp after reduction by ln 2,
// the atanh series for log); sin/cos use the Taylor series after reduction
// to [-pi, pi]. Accuracy is ~1e-15 relative, far below float32 rounding.
#pragma once

#include <cmath>
#include <cstdint>

namespace pierce {
namespace detm {

constexpr double kLn2 = 0.69314718055994530942;
constexpr double kPi = 3.14159265358979323846;
constexpr double kTwoPi = 6.28318530717958647692;

inline double exp(double x) {
    if (x > 700.0) x = 700.0;
    if (x < -700.0) return 0.0;
    double kf = x / kLn2;
    long k = (long)(kf >= 0.0 ? kf + 0.5 : kf - 0.5);
    double r = x - (double)k * kLn2;
    double term = 1.0, sum = 1.0;
    for (int n = 1; n <= 22; ++n) {
        term = term * r / (double)n;
        sum += term;
    }
    return std::ldexp(sum, (int)k);
}

inline double log(double x) {
    if (!(x > 0.0)) return -1e300;
    int e = 0;
    double m = std::frexp(x, &e);  // m in [0.5, 1)
    if (m < 0.70710678118654752) {
        m *= 2.0;
        e -= 1;
    }
    double s = (m - 1.0) / (m + 1.0);
    double s2 = s * s, term = s, sum = 0.0;
    for (int n = 1; n < 61; n += 2) {
        sum += term / (double)n;
        term *= s2;
    }
    return 2.0 * sum + (double)e * kLn2;
}

// Reduce to [-pi, pi] then sum Taylor series.
inline double reduce_angle(double x) {
    double k = std::floor(x / kTwoPi + 0.5);
    return x - k * kTwoPi;
}

inline double sin(double x) {
    x = reduce_angle(x);
    double x2 = x * x, term = x, sum = x;
    for (int n = 1; n <= 20; ++n) {
        term = -term * x2 / (double)((2 * n) * (2 * n + 1));
        sum += term;
    }
    return sum;
}

inline double cos(double x) {
    x = reduce_angle(x);
    double x2 = x * x, term = 1.0, sum = 1.0;
    for (int n = 1; n <= 20; ++n) {
        term = -term * x2 / (double)((2 * n - 1) * (2 * n));
        sum += term;
    }
    return sum;
}

// splitmix64 seeding + xoshiro256** generator (public-domain algorithms by
// Vigna/Blackman, restated).
struct Rng {
    uint64_t s[4];

    static uint64_t splitmix(uint64_t& x) {
        uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (int i = 0; i < 4; ++i) s[i] = splitmix(x);
    }
    static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
    uint64_t next() {
        uint64_t result = rotl(s[1] * 5, 7) * 9;
        uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return result;
    }
    // uniform in [0, 1)
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double lo, double hi) { return lo + (hi - lo) * uniform(); }
    // standard normal via Box-Muller (cosine branch only)
    double normal() {
        double u1 = 1.0 - uniform();  // (0, 1]
        double u2 = uniform();
        return std::sqrt(-2.0 * detm::log(u1)) * detm::cos(kTwoPi * u2);
    }
    uint64_t below(uint64_t n) { return n ? next() % n : 0; }
};

}  // namespace detm
}  // namespace pierce
