// Line profiles of an Allen-Cahn case in the layout of the reference's
// Output_MidX / Output_MidY / Output_Diag (Ark/Cpp/Output.cpp:288-532): five
// zones (Rho, DP = p, TP = thermoPressure, U, V), each
//   variables = <Y|X>,<name>
//   zone T = <name>_M<M_Phi> I = <n>
//   <coordinate>    <value>        (one cell per line)
// along the column nx/2 - 1 (MidX, coordinate y), the row ny/2 - 1 (MidY,
// coordinate x) or the anti-diagonal cells (k, nx - 1 - k), k = 0..nx-1 (Diag,
// coordinate x; needs ny >= nx).  MidX and MidY print with %.20e, Diag with %.8e;
// the zone header's I is ny except in MidY (nx), as the reference writes it.
// File name: <Kind>_Ma<Ma>_<MeshType><NL>_CFL<CFL>ratio_<RhoL/RhoV>step<step>.dat.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace dugks_host {

// fields [ny][nx], cell (i, j) at (i + 1/2, j + 1/2)
struct ProfileFields {
    int nx = 0, ny = 0;
    double m_phi = 0.0;  // the mobility, printed in the zone titles
    std::vector<double> rho, p, tp, u, v;
};

enum class Profile { MidX, MidY, Diag };

std::string format_profile(Profile kind, const ProfileFields &f);  // throws for Diag when ny < nx
// the cells a profile file lists, back into fields of an nx x ny grid (other cells 0);
// throws std::runtime_error on a layout mismatch
ProfileFields read_profile(Profile kind, int nx, int ny, const std::string &path);
Profile profile_kind(const std::string &name);  // "MidX", "MidY", "Diag"
std::string profile_name(Profile kind, const std::string &mach, const std::string &mesh_type, const std::string &nl,
                         const std::string &cfl, double ratio, int64_t step);

}  // namespace dugks_host
