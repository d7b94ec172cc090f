// Line-profile writers (Ark/Cpp/Output.cpp:288-532); layout in profiles.hpp.
#include "profiles.hpp"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace dugks_host {

namespace {

void append(std::string &s, const char *fmt, double a, double b) {
    char buf[96];
    const int n = std::snprintf(buf, sizeof buf, fmt, a, b);
    s.append(buf, (size_t)n);
}

// the grid cell of line k of a profile
void profile_cell(Profile kind, int nx, int ny, int k, int &i, int &j, double &coord) {
    if (kind == Profile::MidX) {
        i = nx / 2 - 1;
        j = k;
        coord = j + 0.5;
    } else if (kind == Profile::MidY) {
        i = k;
        j = ny / 2 - 1;
        coord = i + 0.5;
    } else {
        i = k;
        j = nx - 1 - k;
        coord = i + 0.5;
    }
}

}  // namespace

std::string format_profile(Profile kind, const ProfileFields &f) {
    const int nx = f.nx, ny = f.ny;
    if (kind == Profile::Diag && ny < nx) throw std::runtime_error("Diag profile needs ny >= nx");
    const bool diag = kind == Profile::Diag;
    // the reference sets scientific with 20 digits (8 for Diag) before the first header,
    // so M_Phi in the titles prints the same way
    const char *num = diag ? "%.8e" : "%.20e";
    const std::string row = std::string(num) + "    " + num + "\n";
    const char *axis = kind == Profile::MidY ? "X" : "Y";
    const int count = kind == Profile::MidX ? ny : nx;
    const int zone_i = kind == Profile::MidY ? nx : ny;
    char title[64];
    std::snprintf(title, sizeof title, num, f.m_phi);
    const struct {
        const char *name;
        const std::vector<double> *v;
    } zones[] = {{"Rho", &f.rho}, {"DP", &f.p}, {"TP", &f.tp}, {"U", &f.u}, {"V", &f.v}};
    std::string s;
    for (const auto &z : zones) {
        s += std::string("variables = ") + axis + "," + z.name + "\n";
        s += std::string("zone T = ") + z.name + "_M" + title + " I = " + std::to_string(zone_i) + "\n";
        for (int k = 0; k < count; ++k) {
            int i, j;
            double coord;
            profile_cell(kind, nx, ny, k, i, j, coord);
            append(s, row.c_str(), coord, (*z.v)[(size_t)j * nx + i]);
        }
    }
    return s;
}

Profile profile_kind(const std::string &name) {
    if (name == "MidX") return Profile::MidX;
    if (name == "MidY") return Profile::MidY;
    if (name == "Diag") return Profile::Diag;
    throw std::runtime_error("unknown profile '" + name + "'");
}

ProfileFields read_profile(Profile kind, int nx, int ny, const std::string &path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("cannot open " + path);
    ProfileFields f;
    f.nx = nx;
    f.ny = ny;
    const size_t n = (size_t)nx * ny;
    std::vector<double> *zones[] = {&f.rho, &f.p, &f.tp, &f.u, &f.v};
    const char *names[] = {"Rho", "DP", "TP", "U", "V"};
    const int count = kind == Profile::MidX ? ny : nx;
    std::string line;
    for (int z = 0; z < 5; ++z) {
        zones[z]->assign(n, 0.0);
        if (!std::getline(in, line) || line.rfind("variables = ", 0) != 0) throw std::runtime_error(path + ": no variables line");
        if (!std::getline(in, line)) throw std::runtime_error(path + ": no zone line");
        const std::string head = std::string("zone T = ") + names[z] + "_M";
        if (line.rfind(head, 0) != 0) throw std::runtime_error(path + ": bad zone line '" + line + "'");
        f.m_phi = std::strtod(line.c_str() + head.size(), nullptr);
        for (int k = 0; k < count; ++k) {
            if (!std::getline(in, line)) throw std::runtime_error(path + ": short zone");
            std::istringstream ls(line);
            std::string a, b;
            ls >> a >> b;
            int i, j;
            double coord;
            profile_cell(kind, nx, ny, k, i, j, coord);
            (*zones[z])[(size_t)j * nx + i] = std::strtod(b.c_str(), nullptr);
        }
    }
    return f;
}

std::string profile_name(Profile kind, const std::string &mach, const std::string &mesh_type, const std::string &nl,
                         const std::string &cfl, double ratio, int64_t step) {
    const char *k = kind == Profile::MidX ? "MidX" : (kind == Profile::MidY ? "MidY" : "Diag");
    char r[64];
    std::snprintf(r, sizeof r, "%g", ratio);  // the stream's default format: 6 significant digits
    return std::string(k) + "_Ma" + mach + "_" + mesh_type + nl + "_CFL" + cfl + "ratio_" + r + "step" +
           std::to_string(step) + ".dat";
}

}  // namespace dugks_host
