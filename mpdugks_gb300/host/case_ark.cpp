#include "case_ark.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace dugks_host {

namespace {

std::string trim(const std::string &s) {
    const size_t a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    const size_t b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
}

// the separator the reference writes around '=' (Ark/Cpp/Output.cpp:77-139)
const char *const SEP = "    =    ";
const char *const EXT_RULE = "#----------------GPU----------------";
const char *const END_RULE = "-------------End--------------";

double to_num(const std::string &key, const std::string &v) {
    char *end = nullptr;
    const double x = std::strtod(v.c_str(), &end);
    if (v.empty() || end == v.c_str() || trim(end) != "")
        throw std::runtime_error("Case.ark: entry '" + key + "' is not a number: '" + v + "'");
    return x;
}

}  // namespace

bool CaseArk::has(const std::string &key) const {
    for (const auto &l : lines)
        if (l.entry && l.key == key) return true;
    return false;
}

std::string CaseArk::get(const std::string &key, const std::string &def) const {
    for (const auto &l : lines)
        if (l.entry && l.key == key) return l.value;
    return def;
}

double CaseArk::num(const std::string &key, double def) const {
    if (!has(key)) return def;
    return to_num(key, get(key));
}

void CaseArk::set(const std::string &key, const std::string &value) {
    for (auto &l : lines)
        if (l.entry && l.key == key) {
            l.value = value;
            return;
        }
    // extension block: before the closing rule, opened once
    size_t at = lines.size();
    for (size_t k = 0; k < lines.size(); ++k)
        if (!lines[k].entry && trim(lines[k].text) == END_RULE) at = k;
    bool have_rule = false;
    for (const auto &l : lines)
        if (!l.entry && trim(l.text) == EXT_RULE) have_rule = true;
    Line e;
    e.entry = true;
    e.key = key;
    e.value = value;
    if (!have_rule) {
        Line r;
        r.text = EXT_RULE;
        lines.insert(lines.begin() + at, r);
        ++at;
    }
    lines.insert(lines.begin() + at, e);
}

CaseArk read_case_ark(const std::string &path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("Case.ark: cannot open " + path);
    CaseArk ark;
    std::string s;
    while (std::getline(in, s)) {
        CaseArk::Line l;
        const size_t eq = s.find('=');
        if (eq == std::string::npos) {
            l.text = s;
        } else {
            l.entry = true;
            l.value = trim(s.substr(0, eq));
            l.key = trim(s.substr(eq + 1));
        }
        ark.lines.push_back(l);
    }
    return ark;
}

std::string format_case_ark(const CaseArk &ark) {
    std::string out;
    for (const auto &l : ark.lines) {
        if (l.entry) out += l.value + SEP + l.key;
        else out += l.text;
        out += '\n';
    }
    return out;
}

void write_case_ark(const std::string &path, const CaseArk &ark) {
    std::ofstream o(path, std::ios::binary);
    if (!o) throw std::runtime_error("Case.ark: cannot write " + path);
    o << format_case_ark(ark);
    if (!o) throw std::runtime_error("Case.ark: write failed: " + path);
}

RunConfig config_from_case_ark(const CaseArk &ark) {
    RunConfig c;
    // model: the DmQnName of the reference's velocity models (Ark/Lib/D2Q9AC.cpp:18,
    // Ark/Lib/D2Q9HCZ.cpp:9, Ark/Lib/D2Q9PP.cpp:4, Ark/Lib/D2V16.cpp:9)
    const std::string vm = ark.get("velocity model");
    if (vm == "D2Q9AC") c.cs.model = DUGKS_MODEL_AC;
    else if (vm == "D2Q9Fak" || vm == "D2Q9HCZ") c.cs.model = DUGKS_MODEL_HCZ;
    else if (vm == "D2Q9PP") c.cs.model = DUGKS_MODEL_PP9;
    else if (vm == "D2Q16" || vm == "D2V16") c.cs.model = DUGKS_MODEL_PP16;
    else throw std::runtime_error("Case.ark: unknown velocity model '" + vm + "'");
    const std::string prec = ark.get("precision", "fp64");
    if (prec == "fp64") c.cs.precision = DUGKS_FP64;
    else if (prec == "fp64fma") c.cs.precision = DUGKS_FP64_FMA;
    else if (prec == "fp32dev") c.cs.precision = DUGKS_FP32_DEV;
    else if (prec == "fp64fused") c.cs.precision = DUGKS_FP64_FUSED;
    else throw std::runtime_error("Case.ark: unknown precision '" + prec + "'");
    // grid: "<nx>_<ny>_<type>_<boundary>..." (the reference's mesh file names,
    // Ark/Constant/ZeroFlip.h:47-49)
    c.mesh_name = ark.get("Mesh File");
    {
        int nx = 0, ny = 0;
        char tail[2] = {0};
        if (std::sscanf(c.mesh_name.c_str(), "%d_%d%1c", &nx, &ny, tail) < 2 || nx < 3 || ny < 3)
            throw std::runtime_error("Case.ark: mesh name '" + c.mesh_name + "' does not start with <nx>_<ny>_");
        c.grid.nx = (int)ark.num("nx", nx);
        c.grid.ny = (int)ark.num("ny", ny);
    }
    const std::string bc = ark.get("Boundary Condition");
    c.grid.y_walls = (c.mesh_name.find("Wall") != std::string::npos || bc.find("Wall") != std::string::npos) ? 1 : 0;
    if (ark.has("walls")) c.grid.y_walls = ark.num("walls", 0) != 0 ? 1 : 0;
    // the face reconstruction (OutputCase writes _FLUX_SCHEME_ARK, Ark/Constant/ZeroFlip.h)
    const std::string fs = ark.get("Flux Scheme", "CD");
    if (fs == "CD") c.cs.flux_scheme = DUGKS_FLUX_CD;
    else if (fs == "UW") c.cs.flux_scheme = DUGKS_FLUX_UW;
    else throw std::runtime_error("Case.ark: unknown flux scheme '" + fs + "'");
    // the UW cell gradient (which Grad_VS_* call Ark/Cpp/DUGKS2DSolver.cpp:201-203 keeps;
    // not in OutputCase): 6points (the reference's), LS or 4points
    const std::string gs = ark.get("cell gradient", "6points");
    if (gs == "LS" && c.cs.flux_scheme == DUGKS_FLUX_UW) c.cs.flux_scheme = DUGKS_FLUX_UW_LS;
    else if (gs == "4points" && c.cs.flux_scheme == DUGKS_FLUX_UW) c.cs.flux_scheme = DUGKS_FLUX_UW_4P;
    else if (gs != "6points" && gs != "LS" && gs != "4points")
        throw std::runtime_error("Case.ark: unknown cell gradient '" + gs + "'");
    // the wall treatment (_Wall_3_BCs_BB / _NEE of Ark/Constant/ZeroFlip.h; not in OutputCase)
    const std::string ws = ark.get("wall scheme", "BB");
    if (ws == "BB") c.cs.wall_scheme = DUGKS_WALL_BB;
    else if (ws == "NEE") c.cs.wall_scheme = DUGKS_WALL_NEE;
    else throw std::runtime_error("Case.ark: unknown wall scheme '" + ws + "'");
    c.mesh_type = ark.get("Mesh Type", "Car");
    c.nl = ark.get("NL", std::to_string(c.grid.nx));
    c.mach = ark.get("Mach", "0");
    c.cfl = ark.get("CFL", "0.5");
    c.dt = ark.num("dt", 0.5);
    // the models run at R0 = 1, T0 = 1/3 (Ark/Constant/ZeroReference.h:70); the file's
    // "T0" is that value rounded to 6 digits
    c.T0 = 1.0 / 3.0;
    // constants (names of OutputCase)
    c.cs.Mu0 = ark.num("dynamic viscosity", 0.1);
    c.cs.M_Phi = ark.num("mobility", 0.1);
    c.cs.W = ark.num("inteface width", 5.0);
    c.cs.Sigma = ark.num("Sigma(surface tension coefficient)", 1e-2);
    c.cs.RhoL = ark.num("liquid density", 10.0);
    c.cs.RhoV = ark.num("vapor density", 1.0);
    c.cs.Gy = ark.num("gravity", 0.0);
    c.cs.Tr = ark.num("reduced temperature", 0.85);
    c.cs.aCS = ark.num("a CS", 1.0);
    c.cs.Tc_CS = ark.num("Tc CS", 0.0943);
    c.cs.d2v16_c = ark.num("D2V16 c", 1.2);
    const double chl = ark.num("Characteristic Length", (double)c.grid.nx);
    // run control
    c.residual_stop = ark.num("RESIDUAL", 1e-12);
    const double es = ark.num("End_Step", 0);
    c.end_step = (int64_t)ark.num("steps", es > 0 ? es : 0);
    c.residual_every = (int)ark.num("residual every", 1000);
    c.write_every = (int)ark.num("write every", 10000);
    c.seed = (uint64_t)ark.num("seed", 12345);
    if (c.residual_every < 1 || c.write_every < 1)
        throw std::runtime_error("Case.ark: residual every / write every must be >= 1");
    // initialisation
    c.case_name = ark.get("Case Name");
    std::string init = ark.get("init");
    if (init.empty()) {
        if (c.case_name == "AC_Drop") init = "ac_drop";
        else if (c.case_name == "SCMP_Drop") init = "scmp_drop";
        else throw std::runtime_error("Case.ark: case name '" + c.case_name +
                                      "' has no initialisation here; give an 'init' entry");
    }
    const std::string kinds[] = {"ac_drop", "ac_drop_inside", "ac_rt", "scmp_drop", "pp_noise"};
    c.init_kind = -1;
    for (int k = 0; k < 5; ++k)
        if (init == kinds[k]) c.init_kind = k;
    if (c.init_kind < 0) throw std::runtime_error("Case.ark: unknown init '" + init + "'");
    if (ark.has("init params")) {
        std::stringstream ss(ark.get("init params"));
        std::string tok;
        while (std::getline(ss, tok, ','))
            if (!trim(tok).empty()) c.init_params.push_back(to_num("init params", trim(tok)));
    } else if (c.init_kind <= 1 && ark.has("radius")) {
        c.init_params.push_back(ark.num("radius", 0.36) * chl);  // written as radius / ChLength
    }
    return c;
}

}  // namespace dugks_host
