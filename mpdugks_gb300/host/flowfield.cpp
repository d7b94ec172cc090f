#include "flowfield.hpp"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace dugks_host {

namespace {

struct Section {
    int zone, comps;
    std::vector<double> FlowField::*a;
    std::vector<double> FlowField::*b;
};

const Section SECTIONS[] = {
    {101, 1, &FlowField::rho, nullptr}, {2, 2, &FlowField::u, &FlowField::v}, {1, 1, &FlowField::p, nullptr},
    {3, 1, &FlowField::T, nullptr},     {700, 1, &FlowField::phi, nullptr},   {701, 1, &FlowField::tau, nullptr},
    {702, 1, &FlowField::fx, nullptr},  {703, 1, &FlowField::fy, nullptr},
};

// std::scientific with precision 12, as the reference's output streams
// (Ark/Cpp/Output.cpp:22,52)
void put(std::string &out, double x) {
    char buf[40];
    std::snprintf(buf, sizeof(buf), "%.12e", x);
    out += buf;
}

}  // namespace

std::string format_flowfield(const FlowField &ff) {
    std::string out;
    out.reserve(ff.cells * 9 * 20 + 512);
    for (const auto &s : SECTIONS) {
        const auto &a = ff.*(s.a);
        if (a.size() != ff.cells || (s.b && (ff.*(s.b)).size() != ff.cells))
            throw std::runtime_error("FlowField: a field does not have one value per cell");
        out += "(300 (" + std::to_string(s.zone) + " 2 " + std::to_string(s.comps) + " 0 0 1 " +
               std::to_string(ff.cells) + ")(\n";
        for (size_t n = 0; n < ff.cells; ++n) {
            put(out, a[n]);
            if (s.b) {
                out += "  ";
                put(out, (ff.*(s.b))[n]);
            }
            out += '\n';
        }
        out += "))\n";
    }
    return out;
}

void write_flowfield(const std::string &path, const FlowField &ff) {
    const std::string text = format_flowfield(ff);
    std::ofstream o(path, std::ios::binary);
    if (!o) throw std::runtime_error("FlowField: cannot write " + path);
    o.write(text.data(), (std::streamsize)text.size());
    if (!o) throw std::runtime_error("FlowField: write failed: " + path);
}

FlowField read_flowfield(const std::string &path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("FlowField: cannot open " + path);
    FlowField ff;
    std::string line;
    for (const auto &s : SECTIONS) {
        if (!std::getline(in, line)) throw std::runtime_error("FlowField: missing section " + std::to_string(s.zone));
        int zone = 0, two = 0, comps = 0, z0 = 0, z1 = 0, one = 0;
        long long cells = 0;
        if (std::sscanf(line.c_str(), "(300 (%d %d %d %d %d %d %lld)(", &zone, &two, &comps, &z0, &z1, &one,
                        &cells) != 7 ||
            zone != s.zone || comps != s.comps)
            throw std::runtime_error("FlowField: bad section header '" + line + "'");
        if (ff.cells == 0) ff.cells = (size_t)cells;
        if ((size_t)cells != ff.cells) throw std::runtime_error("FlowField: sections differ in cell count");
        auto &a = ff.*(s.a);
        a.resize(ff.cells);
        if (s.b) (ff.*(s.b)).resize(ff.cells);
        for (size_t n = 0; n < ff.cells; ++n) {
            if (!std::getline(in, line)) throw std::runtime_error("FlowField: truncated section");
            char *end = nullptr;
            a[n] = std::strtod(line.c_str(), &end);
            if (s.b) (ff.*(s.b))[n] = std::strtod(end, &end);
        }
        if (!std::getline(in, line) || line != "))") throw std::runtime_error("FlowField: section not closed");
    }
    return ff;
}

std::string flowfield_name(int64_t step, double t, const std::string &mach, const std::string &mesh_type,
                           const std::string &nl, const std::string &cfl) {
    // default stream formatting of the time, as the reference's file name
    // (Ark/Cpp/Output.cpp:543-545)
    std::ostringstream o;
    o << "step" << step << "Ma" << mach << "_" << mesh_type << nl << "_CFL" << cfl << "_T" << t << ".dat";
    return o.str();
}

}  // namespace dugks_host
