// Command-line options of the query executables.  The flags, defaults and
// lenient parsing (unknown arguments ignored, a flag missing its value is
// ignored) follow pierce/query/src/applications/app_cli_options.h:10-163 and
// each application's options class.
#pragma once

#include <string>
#include <utility>
#include <vector>

struct CliBase {
    using Entry = std::pair<std::string, std::string>;
    virtual ~CliBase() = default;

    bool help = false;
    std::string mesh1, mesh2, output_json, ptx;
    int runs = 1, warmup_runs = 2;
    bool export_results = true;
    bool allow_no_export = false;
    bool has_runs = true;

    explicit CliBase(std::string default_json) : output_json(std::move(default_json)) {}
    void parse(int argc, char** argv);
    void sanitize() {
        if (runs < 1) runs = 1;
        if (warmup_runs < 0) warmup_runs = 0;
    }
    bool has_meshes() const { return !mesh1.empty() && !mesh2.empty(); }

    static void print_help(const char* exe, const std::string& usage, const std::string& description,
                           const std::vector<Entry>& options);
    void common_help(std::vector<Entry>& o, const std::string& m1 = "Path to first mesh dataset (geometry file)",
                     const std::string& m2 = "Path to second mesh dataset (geometry file)") const;

protected:
    // returns true if consumed
    virtual bool app_option(const std::string& arg, int& i, int argc, char** argv) {
        (void)arg, (void)i, (void)argc, (void)argv;
        return false;
    }
};
