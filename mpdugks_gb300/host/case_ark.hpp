// Case.ark: the reference's case description (written by OutputCase,
// Ark/Cpp/Output.cpp:65-141) read as the configuration of a GPU run.
//
// Layout: one entry per line, "<value>    =    <key>", in the reference's
// order; lines without '=' are section rules ("#----...", "-----...") or
// blank.  The reader keeps every line, so a file it read is written back
// byte for byte; values set afterwards replace the text of their line.
// Keys this library adds (precision, gravity, init, ...) go in a block of
// their own before the closing rule.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/dugks_gpu.h"

namespace dugks_host {

struct CaseArk {
    struct Line {
        bool entry = false;
        std::string key, value, text;  // text: the whole line when !entry
    };
    std::vector<Line> lines;

    bool has(const std::string &key) const;
    std::string get(const std::string &key, const std::string &def = "") const;
    double num(const std::string &key, double def) const;
    // replace the value of an existing entry, or add it to the extension block
    void set(const std::string &key, const std::string &value);
};

CaseArk read_case_ark(const std::string &path);  // throws std::runtime_error
void write_case_ark(const std::string &path, const CaseArk &ark);
std::string format_case_ark(const CaseArk &ark);

// What a run needs, decoded from a Case.ark.
struct RunConfig {
    dugks_case_t cs{};
    dugks_grid_t grid{};
    int init_kind = 0;               // dugks_gpu_init kind
    std::vector<double> init_params;
    uint64_t seed = 12345;
    int64_t end_step = 0;
    double residual_stop = 1e-12;    // RESIDUAL
    int residual_every = 1000;       // ResidualControl (Ark/Constant/ZeroNamespace.h:175)
    int write_every = 10000;         // writeFileControl (Ark/Constant/ZeroNamespace.h:177)
    double dt = 0.5, T0 = 1.0 / 3.0;
    std::string case_name, mesh_name, mesh_type = "Car", mach = "0", cfl = "0.5", nl;
};

// Decode: velocity model (D2Q9AC, D2Q9Fak = HCZ, D2Q9PP, D2Q16), grid size
// and wall kind from the mesh name "<nx>_<ny>_<type>_<Periodic|Wall>...",
// the phase-field constants, End_Step / RESIDUAL; the case name selects the
// initialisation (AC_Drop, SCMP_Drop) unless "init" is given.  Throws
// std::runtime_error for a missing or invalid entry.
RunConfig config_from_case_ark(const CaseArk &ark);

}  // namespace dugks_host
