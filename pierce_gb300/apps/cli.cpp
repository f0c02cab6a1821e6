#include "cli.h"

#include <cstdlib>
#include <iomanip>
#include <iostream>

void CliBase::parse(int argc, char** argv) {
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--help" || a == "-h") {
            help = true;
        } else if (a == "--mesh1" && i + 1 < argc) {
            mesh1 = argv[++i];
        } else if (a == "--mesh2" && i + 1 < argc) {
            mesh2 = argv[++i];
        } else if (a == "--output" && i + 1 < argc) {
            output_json = argv[++i];
        } else if (a == "--ptx" && i + 1 < argc) {
            ptx = argv[++i];  // accepted for compatibility; no PTX is loaded
        } else if (has_runs && a == "--runs" && i + 1 < argc) {
            runs = std::atoi(argv[++i]);
        } else if (has_runs && a == "--warmup-runs" && i + 1 < argc) {
            warmup_runs = std::atoi(argv[++i]);
        } else if (allow_no_export && a == "--no-export") {
            export_results = false;
        } else {
            app_option(a, i, argc, argv);
        }
    }
}

void CliBase::print_help(const char* exe, const std::string& usage, const std::string& description,
                         const std::vector<Entry>& options) {
    std::cout << "Usage: " << exe << " " << usage << std::endl;
    if (!description.empty()) std::cout << description << std::endl;
    std::cout << "Options:" << std::endl;
    for (const auto& e : options) std::cout << "  " << std::left << std::setw(34) << e.first << e.second << std::endl;
}

void CliBase::common_help(std::vector<Entry>& o, const std::string& m1, const std::string& m2) const {
    o.emplace_back("--mesh1 <path>", m1);
    o.emplace_back("--mesh2 <path>", m2);
    o.emplace_back("--output <path>", "Path to JSON file for performance timing output");
    o.emplace_back("--ptx <path>", "Accepted for compatibility (no PTX is used)");
    if (has_runs) {
        o.emplace_back("--runs <number>", "Number of measured query runs (default: 1)");
        o.emplace_back("--warmup-runs <number>", "Number of warmup iterations (default: 2)");
    }
}
