// Phase timer whose stdout table and JSON file follow the reference's
// PerformanceTimer (pierce/query/src/timer.h:9-49, timer.cpp): sequential
// phases (start/next/finish), extra measurements added by name, counters,
// and a JSON file {"phases": {"<lowercased name>_<k>": {"duration_us",
// "duration_ms"}}, "counters": {...}, "total": {...}} that the benchmark
// adapters parse.
#pragma once

#include <chrono>
#include <string>
#include <vector>

class PhaseTimer {
public:
    void start(const std::string& name);
    void next(const std::string& name);
    void finish(const std::string& json_path);
    void add_measurement(const std::string& name, long long duration_us);
    void add_counter(const std::string& name, unsigned long long value);
    long long total_us() const;

private:
    using clock = std::chrono::high_resolution_clock;
    struct Phase {
        std::string name;
        clock::time_point begin, end;
        long long us = 0;
        bool closed = false;
    };
    std::vector<Phase> phases_, measurements_;
    std::vector<std::pair<std::string, unsigned long long>> counters_;
    clock::time_point t0_, t1_;
    bool running_ = false, finished_ = false;
    void close_current();
    void print() const;
    void write_json(const std::string& path) const;
};
