#include "mesh_cas.hpp"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace dugks_host {

namespace {

[[noreturn]] void fail(const std::string &m) { throw std::runtime_error(".cas: " + m); }

// node coordinates are rounded to 1e-10, as the reference's validDigits
// (Ark/Lib/MeshConstructFunc.h:57-60 with digits = 1e10)
double round10(double v) { return std::round(v * 1e10) / 1e10; }

// whitespace-separated tokens of the lines after a header, across lines
struct Body {
    const std::vector<std::string> &lines;
    size_t line;
    std::istringstream cur;
    Body(const std::vector<std::string> &l, size_t next) : lines(l), line(next) { cur.str(""); }
    bool token(std::string &t) {
        while (!(cur >> t)) {
            if (line >= lines.size()) return false;
            cur.clear();
            cur.str(lines[line++]);
        }
        return true;
    }
    long hex(const char *what) {
        std::string t;
        if (!token(t)) fail(std::string("file ends inside the ") + what + " section");
        char *end = nullptr;
        const long v = std::strtol(t.c_str(), &end, 16);
        if (end == t.c_str() || *end) fail(std::string("bad hexadecimal '") + t + "' in the " + what + " section");
        return v;
    }
    double num(const char *what) {
        std::string t;
        if (!token(t)) fail(std::string("file ends inside the ") + what + " section");
        char *end = nullptr;
        const double v = std::strtod(t.c_str(), &end);
        if (end == t.c_str() || *end) fail(std::string("bad number '") + t + "' in the " + what + " section");
        return v;
    }
};

int cell_type_of(long elem) {
    if (elem == 3) return 4;  // quadrilateral
    if (elem == 1) return 3;  // triangle
    fail("element type " + std::to_string(elem) + " is not a 2D cell");
}

const char *bc_name(int bc) {
    switch (bc) {
        case 2: return "interior";
        case 3: return "wall";
        case 4: return "pressure inlet";
        case 5: return "pressure outlet";
        case 7: return "symmetry";
        case 8: return "periodic shadow";
        case 9: return "pressure far field";
        case 10: return "velocity inlet";
        case 12: return "periodic";
        default: return "unknown";
    }
}

}  // namespace

CasMesh parse_cas(const std::string &text) {
    std::vector<std::string> lines;
    {
        std::istringstream in(text);
        std::string l;
        while (std::getline(in, l)) lines.push_back(l);
    }
    CasMesh m;
    int nodes = -1, faces = -1;
    for (size_t li = 0; li < lines.size(); ++li) {
        std::string s = lines[li];
        if (s.empty() || s.front() != '(') continue;
        while (!s.empty() && std::isspace((unsigned char)s.back())) s.pop_back();
        const bool body = !s.empty() && s.back() == '(';
        std::string flat;
        for (char ch : s)
            if (ch != '(' && ch != ')') flat += ch;
        std::istringstream hs(flat);
        int index = 0;
        if (!(hs >> index) || !(index == 10 || index == 12 || index == 13 || index == 18)) continue;
        std::vector<long> h;
        std::string t;
        while (hs >> t) {
            char *end = nullptr;
            const long v = std::strtol(t.c_str(), &end, 16);
            if (end == t.c_str() || *end) break;  // a zone name or other text ends the numbers
            h.push_back(v);
        }
        if (index == 18) {
            if (!body) continue;
            if (h.size() < 2) fail("periodic section header without a face range");
            Body b(lines, li + 1);
            for (long k = h[0]; k <= h[1]; ++k) {
                const long f0 = b.hex("periodic"), f1 = b.hex("periodic");
                m.periodic.push_back({(int)f0 - 1, (int)f1 - 1});
            }
            li = b.line - 1;
            continue;
        }
        if (h.size() < 3) fail("section " + std::to_string(index) + " header has too few numbers");
        const long zone = h[0], first = h[1], last = h[2];
        if (last < first - 1 || first < 0 || last > (1L << 30)) fail("bad id range in section " + std::to_string(index));
        if (index == 10) {
            if (zone == 0 || !body) {
                nodes = (int)last;
                m.x.assign(nodes, 0.0);
                m.y.assign(nodes, 0.0);
                continue;
            }
            if (nodes < 0 || last > nodes) fail("node body outside the declared node count");
            Body b(lines, li + 1);
            for (long k = first - 1; k < last; ++k) {
                m.x[k] = round10(b.num("node"));
                m.y[k] = round10(b.num("node"));
            }
            li = b.line - 1;
        } else if (index == 12) {
            if (zone == 0) {
                m.ncells = (int)last;
                m.cell_type.assign(m.ncells, 0);
                continue;
            }
            if (m.ncells <= 0 || last > m.ncells) fail("cell zone outside the declared cell count");
            if (!body) {
                if (h.size() < 5) fail("cell zone header without an element type");
                const int ct = cell_type_of(h[4]);
                for (long k = first - 1; k < last; ++k) m.cell_type[k] = ct;
            } else {
                Body b(lines, li + 1);
                for (long k = first - 1; k < last; ++k) m.cell_type[k] = cell_type_of(b.hex("cell"));
                li = b.line - 1;
            }
        } else {  // 13
            if (zone == 0 || !body) {
                faces = (int)last;
                m.faces.assign(faces, CasMesh::Face{});
                continue;
            }
            if (faces < 0 || last > faces) fail("face body outside the declared face count");
            if (h.size() < 5) fail("face zone header without bc and face types");
            const int bc = (int)h[3], ft = (int)h[4];
            if (ft != 0 && ft != 2) fail("face type " + std::to_string(ft) + " is not a 2D line face");
            Body b(lines, li + 1);
            for (long k = first - 1; k < last; ++k) {
                if (ft == 0 && b.hex("face") != 2) fail("a mixed-type face with other than two nodes");
                CasMesh::Face f;
                f.n0 = (int)b.hex("face") - 1;
                f.n1 = (int)b.hex("face") - 1;
                f.c0 = (int)b.hex("face") - 1;
                f.c1 = (int)b.hex("face") - 1;
                f.bc = bc;
                f.zone = (int)zone;
                m.faces[k] = f;
            }
            li = b.line - 1;
        }
    }
    if (nodes <= 0 || m.ncells <= 0 || faces <= 0) fail("missing node, cell or face declarations");
    for (size_t k = 0; k < m.faces.size(); ++k) {
        const auto &f = m.faces[k];
        if (f.n0 < 0 || f.n0 >= nodes || f.n1 < 0 || f.n1 >= nodes || f.c0 < 0 || f.c0 >= m.ncells ||
            f.c1 < -1 || f.c1 >= m.ncells)
            fail("face " + std::to_string(k + 1) + " refers to a missing node or cell");
    }
    for (const auto &p : m.periodic)
        if (p.first < 0 || p.first >= faces || p.second < 0 || p.second >= faces) fail("periodic pair of missing faces");
    return m;
}

CasMesh read_cas(const std::string &path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("cannot open mesh file " + path);
    std::stringstream ss;
    ss << in.rdbuf();
    return parse_cas(ss.str());
}

CartesianMap cartesian_map(const CasMesh &m) {
    const double eps = 1e-9;
    const int nc = m.ncells;
    for (int k = 0; k < nc; ++k)
        if (m.cell_type[k] != 4) fail("cell " + std::to_string(k + 1) + " is not a quadrilateral");
    std::vector<int> nfaces(nc, 0);
    std::vector<double> cx(nc, 0.0), cy(nc, 0.0);
    double xmin = m.x[0], ymin = m.y[0];
    for (size_t k = 0; k < m.x.size(); ++k) {
        xmin = std::min(xmin, m.x[k]);
        ymin = std::min(ymin, m.y[k]);
    }
    // unit, axis-aligned faces; cell centre = mean of its four face midpoints
    for (size_t k = 0; k < m.faces.size(); ++k) {
        const auto &f = m.faces[k];
        const double dx = m.x[f.n1] - m.x[f.n0], dy = m.y[f.n1] - m.y[f.n0];
        if (std::fabs(std::hypot(dx, dy) - 1.0) > eps || (std::fabs(dx) > eps && std::fabs(dy) > eps))
            fail("face " + std::to_string(k + 1) + " is not an axis-aligned face of length 1 (the GPU path takes "
                 "unit square cells)");
        const double mx = 0.5 * (m.x[f.n0] + m.x[f.n1]), my = 0.5 * (m.y[f.n0] + m.y[f.n1]);
        for (int c : {f.c0, f.c1})
            if (c >= 0) {
                nfaces[c] += 1;
                cx[c] += 0.25 * mx;
                cy[c] += 0.25 * my;
            }
    }
    CartesianMap map;
    std::vector<int> ii(nc), jj(nc);
    for (int k = 0; k < nc; ++k) {
        if (nfaces[k] != 4) fail("cell " + std::to_string(k + 1) + " has " + std::to_string(nfaces[k]) + " faces");
        const double fi = cx[k] - xmin - 0.5, fj = cy[k] - ymin - 0.5;
        ii[k] = (int)std::lround(fi);
        jj[k] = (int)std::lround(fj);
        if (std::fabs(fi - ii[k]) > eps || std::fabs(fj - jj[k]) > eps)
            fail("cell " + std::to_string(k + 1) + " is off the unit grid");
        map.nx = std::max(map.nx, ii[k] + 1);
        map.ny = std::max(map.ny, jj[k] + 1);
    }
    if ((long long)map.nx * map.ny != nc) fail("the cells do not fill a rectangle");
    map.cell_index.assign(nc, -1);
    std::vector<int> seen((size_t)nc, 0);
    for (int k = 0; k < nc; ++k) {
        const int idx = jj[k] * map.nx + ii[k];
        if (seen[idx]++) fail("two cells share a position");
        map.cell_index[k] = idx;
    }
    // orientation: the normal (dy, -dx) of n0 -> n1 points from the owner out
    // (Ark/Cpp/Mesh/Face_2D.cpp, checked by Ark/Cpp/Mesh/MeshCartesian.cpp:131-248);
    // interior faces join neighbouring cells; boundary faces by side
    enum { LEFT, RIGHT, BOTTOM, TOP };
    std::vector<int> side(m.faces.size(), -1), line(m.faces.size(), -1);
    int ybc = -1;
    for (size_t k = 0; k < m.faces.size(); ++k) {
        const auto &f = m.faces[k];
        const int nxv = (int)std::lround(m.y[f.n1] - m.y[f.n0]), nyv = (int)std::lround(m.x[f.n0] - m.x[f.n1]);
        const double mx = 0.5 * (m.x[f.n0] + m.x[f.n1]), my = 0.5 * (m.y[f.n0] + m.y[f.n1]);
        if (std::fabs(mx - cx[f.c0] - 0.5 * nxv) > eps || std::fabs(my - cy[f.c0] - 0.5 * nyv) > eps)
            fail("face " + std::to_string(k + 1) + ": its normal does not point out of its owner cell");
        const std::string fk = "face " + std::to_string(k + 1) + " (" + bc_name(f.bc) + ", bc_type " +
                               std::to_string(f.bc) + ")";
        if (f.c1 >= 0) {
            if (f.bc != 2) fail(fk + " joins two cells but is not interior");
            if (ii[f.c1] != ii[f.c0] + nxv || jj[f.c1] != jj[f.c0] + nyv)
                fail(fk + " does not join neighbouring cells");
            continue;
        }
        if (f.bc == 2) fail(fk + " is interior without a neighbour cell");
        const bool periodic = f.bc == 12 || f.bc == 8;
        if (nxv != 0) {
            side[k] = nxv < 0 ? LEFT : RIGHT;
            line[k] = jj[f.c0];
            if ((side[k] == LEFT && ii[f.c0] != 0) || (side[k] == RIGHT && ii[f.c0] != map.nx - 1))
                fail(fk + " is a boundary face inside the domain");
            if (!periodic) fail(fk + " on an x boundary: the GPU path takes periodic x boundaries");
        } else {
            side[k] = nyv < 0 ? BOTTOM : TOP;
            line[k] = ii[f.c0];
            if ((side[k] == BOTTOM && jj[f.c0] != 0) || (side[k] == TOP && jj[f.c0] != map.ny - 1))
                fail(fk + " is a boundary face inside the domain");
            const int kind = periodic ? 12 : f.bc;
            if (kind != 12 && kind != 3)
                fail(fk + " on a y boundary: the GPU path takes periodic or wall y boundaries");
            if (ybc >= 0 && ybc != kind) fail("the y boundaries mix periodic and wall faces");
            ybc = kind;
        }
    }
    map.y_walls = ybc == 3 ? 1 : 0;
    // every periodic face paired once, with the face across the domain on the same row / column
    std::vector<int> paired(m.faces.size(), 0);
    for (const auto &p : m.periodic) {
        const int a = p.first, b = p.second;
        const bool ok = side[a] >= 0 && side[b] >= 0 && line[a] == line[b] &&
                        ((side[a] == LEFT && side[b] == RIGHT) || (side[a] == RIGHT && side[b] == LEFT) ||
                         (side[a] == BOTTOM && side[b] == TOP) || (side[a] == TOP && side[b] == BOTTOM));
        if (!ok) fail("periodic pair (" + std::to_string(a + 1) + ", " + std::to_string(b + 1) +
                      ") does not join opposite boundary faces of one row or column");
        paired[a] += 1;
        paired[b] += 1;
    }
    for (size_t k = 0; k < m.faces.size(); ++k) {
        const bool periodic = m.faces[k].c1 < 0 && (m.faces[k].bc == 12 || m.faces[k].bc == 8);
        if (periodic && paired[k] != 1)
            fail("periodic face " + std::to_string(k + 1) + " is in " + std::to_string(paired[k]) + " pairs");
    }
    return map;
}

std::vector<double> to_mesh_order(const CartesianMap &map, const std::vector<double> &row_major) {
    std::vector<double> out(map.cell_index.size());
    for (size_t k = 0; k < out.size(); ++k) out[k] = row_major[(size_t)map.cell_index[k]];
    return out;
}

}  // namespace dugks_host
