// Fluent-style .cas mesh files, the reference's mesh input
// (MeshConstruct, Ark/Cpp/Mesh/MeshConstruct.cpp:69-123, section handlers
// in Ark/Lib/MeshConstructFunc.h), read as the grid of a GPU run.
//
// Text layout the reference accepts and this reader follows: only lines that
// start with '(' are headers; parentheses are dropped, the first number is the
// section index (decimal), the rest are hexadecimal; a header whose last
// non-blank character is '(' is followed by a body.  Sections: 10 nodes
// (decimal "x y" pairs, rounded to 1e-10 like the reference), 12 cells
// (element type 3 quad / 1 triangle, in the header or one per cell in a body),
// 13 faces ("n0 n1 c0 c1", or "2 n0 n1 c0 c1" for face type 0; bc_type 2
// interior, 12/8 periodic/shadow, 3 wall, 4/5 pressure inlet/outlet,
// 7 symmetry, 9 far field, 10 velocity inlet), 18 periodic face pairs.
// Other sections are skipped.
//
// The GPU path runs uniform Cartesian meshes of unit square cells, periodic
// in x and periodic or walled in y.  cartesian_map() checks that a mesh is
// one and gives each of its cells (the reference's CellArray order, which is
// the order of FlowField output) its place j*nx + i in the GPU's row-major
// fields.
#pragma once

#include <string>
#include <vector>

namespace dugks_host {

struct CasMesh {
    struct Face {
        int n0 = -1, n1 = -1;  // nodes, 0-based
        int c0 = -1, c1 = -1;  // owner and neighbour cells, 0-based; c1 = -1 on a boundary
        int bc = 0, zone = 0;
    };
    std::vector<double> x, y;  // node coordinates
    int ncells = 0;
    std::vector<int> cell_type;  // 4 quad, 3 triangle (the reference's celltype)
    std::vector<Face> faces;
    std::vector<std::pair<int, int>> periodic;  // face pairs, 0-based
};

CasMesh read_cas(const std::string &path);  // throws std::runtime_error
CasMesh parse_cas(const std::string &text);

struct CartesianMap {
    int nx = 0, ny = 0, y_walls = 0;
    std::vector<int> cell_index;  // mesh cell k -> j*nx + i
};

// Throws std::runtime_error naming what the GPU path does not take (cell
// shape, size, boundary type, unpaired periodic face, face orientation).
CartesianMap cartesian_map(const CasMesh &m);

// a field in the GPU's row-major order -> the mesh's cell order
std::vector<double> to_mesh_order(const CartesianMap &map, const std::vector<double> &row_major);

}  // namespace dugks_host
