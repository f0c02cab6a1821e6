#include "timer.h"

#include <cctype>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>

static std::string lower(const std::string& s) {
    std::string o;
    o.reserve(s.size());
    for (char c : s) o.push_back((char)std::tolower((unsigned char)c));
    return o;
}

void PhaseTimer::start(const std::string& name) {
    phases_.clear();
    measurements_.clear();
    counters_.clear();
    t0_ = clock::now();
    running_ = true;
    finished_ = false;
    phases_.push_back(Phase{name, t0_, {}, 0, false});
}

void PhaseTimer::close_current() {
    if (!phases_.empty() && !phases_.back().closed) {
        Phase& p = phases_.back();
        p.end = clock::now();
        p.us = std::chrono::duration_cast<std::chrono::microseconds>(p.end - p.begin).count();
        p.closed = true;
    }
}

void PhaseTimer::next(const std::string& name) {
    if (!running_) {
        std::cerr << "Timer not started! Call start() first." << std::endl;
        return;
    }
    close_current();
    phases_.push_back(Phase{name, clock::now(), {}, 0, false});
}

void PhaseTimer::add_measurement(const std::string& name, long long duration_us) {
    Phase p;
    p.name = name;
    p.us = duration_us;
    p.closed = true;
    measurements_.push_back(p);
}

void PhaseTimer::add_counter(const std::string& name, unsigned long long value) { counters_.emplace_back(name, value); }

long long PhaseTimer::total_us() const {
    if (!finished_) return -1;
    return std::chrono::duration_cast<std::chrono::microseconds>(t1_ - t0_).count();
}

void PhaseTimer::finish(const std::string& json_path) {
    if (!running_) {
        std::cerr << "Timer not started! Call start() first." << std::endl;
        return;
    }
    close_current();
    t1_ = clock::now();
    running_ = false;
    finished_ = true;
    print();
    write_json(json_path);
}

void PhaseTimer::print() const {
    std::cout << "\n=== Detailed Performance Summary ===" << std::endl;
    auto row = [](const Phase& p) {
        std::cout << std::left << std::setw(30) << (p.name + ":") << std::right << std::setw(20) << p.us
                  << " microseconds (" << std::fixed << std::setprecision(2) << (double)p.us / 1000.0 << " ms)"
                  << std::endl;
    };
    for (const auto& p : phases_) row(p);
    for (const auto& p : measurements_) row(p);
    if (!counters_.empty()) {
        std::cout << "\n=== Profiling Counters ===" << std::endl;
        for (const auto& c : counters_)
            std::cout << std::left << std::setw(30) << (c.first + ":") << std::right << std::setw(20) << c.second
                      << std::endl;
    }
    const long long t = total_us();
    if (t > 0)
        std::cout << std::left << std::setw(25) << "Total Execution Time:" << std::right << std::setw(10) << t
                  << " microseconds (" << std::fixed << std::setprecision(2) << (double)t / 1000.0 << " ms)"
                  << std::endl;
    std::cout.unsetf(std::ios::floatfield);
}

void PhaseTimer::write_json(const std::string& path) const {
    std::ofstream f(path);
    if (!f) {
        std::cerr << "Warning: Could not write timing results to file." << std::endl;
        return;
    }
    std::vector<const Phase*> all;
    for (const auto& p : phases_) all.push_back(&p);
    for (const auto& p : measurements_) all.push_back(&p);
    std::map<std::string, int> seen;
    f << "{\n  \"phases\": {\n";
    for (size_t i = 0; i < all.size(); ++i) {
        const std::string key = lower(all[i]->name);
        const int k = ++seen[key];
        f << "    \"" << key << "_" << k << "\": {\n";
        f << "      \"duration_us\": " << all[i]->us << ",\n";
        char ms[64];
        std::snprintf(ms, sizeof(ms), "%.2f", (double)all[i]->us / 1000.0);
        f << "      \"duration_ms\": " << ms << "\n    }" << (i + 1 < all.size() ? "," : "") << "\n";
    }
    f << "  },\n  \"counters\": {\n";
    for (size_t i = 0; i < counters_.size(); ++i)
        f << "    \"" << lower(counters_[i].first) << "\": " << counters_[i].second
          << (i + 1 < counters_.size() ? "," : "") << "\n";
    f << "  },\n";
    const long long t = total_us();
    if (t > 0) {
        char ms[64];
        std::snprintf(ms, sizeof(ms), "%.2f", (double)t / 1000.0);
        f << "  \"total\": {\n    \"duration_us\": " << t << ",\n    \"duration_ms\": " << ms << "\n  }\n";
    } else {
        f << "  \"total\": null\n";
    }
    f << "}\n";
    std::cout << "Performance timing written to " << path << std::endl;
}
