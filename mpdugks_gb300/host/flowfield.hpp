// FlowField output in the layout of the reference's Output_Flowfield
// (Ark/Cpp/Output.cpp:541-606): for each field a section
//   (300 (<zone> 2 <components> 0 0 1 <cells>)(
//   <one cell per line, %.12e, components separated by two spaces>
//   ))
// with zones rho 101, (u v) 2, p 1, T 3, phi 700, tau 701, Fx 702, Fy 703,
// cells in the reference's CellArray order (cell (i, j) of a generated
// Cartesian mesh is cell j*nx + i), and the file name
// step<step>Ma<Ma>_<MeshType><NL>_CFL<CFL>_T<t>.dat.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace dugks_host {

struct FlowField {
    size_t cells = 0;
    std::vector<double> rho, u, v, p, T, phi, tau, fx, fy;
};

std::string format_flowfield(const FlowField &ff);
void write_flowfield(const std::string &path, const FlowField &ff);
FlowField read_flowfield(const std::string &path);  // throws std::runtime_error
std::string flowfield_name(int64_t step, double t, const std::string &mach, const std::string &mesh_type,
                           const std::string &nl, const std::string &cfl);

}  // namespace dugks_host
