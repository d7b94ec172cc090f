// Device-side definitions shared by the DUGKS kernels (sm_103a).
//
// Grid: nx*ny unit cells, SoA fields [ny][pitch] (pitch = nx rounded up to 32
// doubles = 256 B, so every row starts on a 256-byte boundary and a warp's 32
// consecutive cells are one coalesced 256-B access).  x is periodic; y is
// periodic or closed by bounce-back walls with one extrapolated ghost row on
// each side (Ark/Cpp/Boundary.cpp:38-139), evaluated on the fly.
//
// Face numbering: x-face (i,j) is the west face of cell (i,j), between
// (i-1,j) and (i,j), normal +x; y-face (i,j) is the south face of cell
// (i,j), between (i,j-1) and (i,j), normal +y; with walls y-faces run
// j = 0..ny (0 and ny are the wall faces).  The reference evaluates each
// face from its owner's side and each periodic face twice
// (Ark/Cpp/DUGKS2DSolver.cpp:219-230); its central-difference face formulas
// are orientation independent, so every physical face is evaluated once here.
#pragma once
#include <cstddef>
#include <cstdint>

namespace dugks {

enum Model { AC = 0, HCZ = 1, PP9 = 2, PP16 = 3 };

enum Field {
    F_RHO = 0, F_U, F_V, F_P, F_PHI, F_TAU, F_PHIX, F_PHIY, F_RHOX, F_RHOY, F_FX, F_FY,
    F_PPU, F_PPV, F_PSI, F_SCG, NFIELDS
};

// Constants of one case.  Names follow Ark/Constant/ZeroReference.h and
// Ark/Constant/ZeroNamespace.h; all are derived on the host with the
// reference's expressions (see host_params.cpp).
struct Params {
    int nx, ny, pitch, walls, model, gravity, Q, nee;  // nee: NEE wall faces (DUGKS_WALL_NEE)
    double R0, T0, RT, Lambda0, dt, hDt, Tau0, Kp, MinL, dx, dy, _2dx, _2dy;
    double aPhi, bPhi, Beta, Kappa, wI, PhiL, PhiV, RhoL, RhoV, Gy, NuL, NuV, TauMass;
    double h_aBP, h_bBP, h_cBP, h_ah, h_bh, h_ch;  // constant phase-field relaxation factors
    double aTP, bTP, dtV;                          // 4/3, 1/3, dt/volume
    double T_CS, aCS;                              // Carnahan-Starling EOS
    // Reconstruction denominators as multipliers: -1/dx, -1/dy, 1/(2dy), 1/(-2dx).
    // grad_mul = 1 when dx and dy are powers of two, so x/d == x*(1/d) exactly.
    double r_ndx, r_ndy, r_2dy, r_n2dx;
    // reciprocals RN(1/d) of divisors fixed per case, for the correctly rounded quotient
    // qdiv_rn: 1/RT, 1/(6 2dx), 1/(6 2dy), 1/(6 MinL MinL), 1/(W (PhiL - PhiV)), 1/(RT dt)
    double r_RT, r_g6x, r_g6y, r_lap, r_wI, r_RTdt;
    int grad_mul, uw;                              // uw: upwind face reconstruction (DUGKS_FLUX_UW*)
    int uw_grad;                                   // its cell gradient: 0 6-point, 1 least squares, 2 4-point
    double c16;                                    // D2V16 lattice speed
    // D2V16 inverse moment matrix of this case, [16][16] in the case's device memory
    // (Ark/Lib/D2V16.cpp:34-52): each case holds its own
    const double *iM16;
    double xi_u[16], xi_v[16], omega[16];
    int bb[16];
};

// Device pointers of one case.  qs = ny*pitch (stride between velocities).
struct State {
    double *f, *h;             // tilde distributions [Q][ny][pitch]
    double *bf, *bh;           // BarP (collision pre-step) [Q][ny][pitch]
    double *xff, *xfh;         // x-face fluxes [Q][ny][pitch]
    double *yff, *yfh;         // y-face fluxes [Q][ny+1][pitch]
    double *fld[NFIELDS];      // macroscopic cell fields [ny][pitch]
    double *gphi;              // 2 buffers x (bottom, top) ghost phi rows [2][2][pitch]
    // pseudopotential face state, x: [ny][pitch], y: [ny][pitch] (periodic only)
    double *xfFx, *xfFy, *yfFx, *yfFy;
    double *xpsi, *ypsi, *xscg, *yscg, *xrho, *yrho, *xu, *yu, *xv, *yv;
    double *xbf, *ybf;         // face BhDt kept between the two pseudopotential face passes [Q][ny][pitch]
    double *gfx, *gfy, *ghx, *ghy;  // UW: cell gradients of f-bar-plus and h-bar-plus [Q][ny][pitch]
    // UW: fluxes of the periodic boundary faces as the reference's low-side faces (owner
    // inside at column 0 / row 0): x [Q][ny] (stride ny), y [Q][pitch] (stride pitch)
    double *xlo_f, *xlo_h, *ylo_f, *ylo_h;
    // NEE walls: equilibria and sources of the wall rows, [4: fEq, fSo, hEq, hSo][2: bottom, top][Q][pitch]
    double *weq;
    size_t qs, qsy;            // velocity strides of cell/x-face arrays and of y-face arrays
};

// D2Q9 velocity set (Ark/Lib/D2Q9.h:86-90), MaSpan = sqrt(3RT) = 1 exactly.
__host__ __device__ constexpr int d2q9_xu(int q) { return q == 1 || q == 2 || q == 8 ? 1 : (q >= 4 && q <= 6 ? -1 : 0); }
__host__ __device__ constexpr int d2q9_xv(int q) { return q >= 2 && q <= 4 ? 1 : (q >= 6 ? -1 : 0); }
__host__ __device__ constexpr double d2q9_w(int q) {
    return q == 0 ? 4.0 / 9.0 : ((q & 1) ? 1.0 / 9.0 : 1.0 / 36.0);
}
__host__ __device__ constexpr int d2q9_bb(int q) { return q == 0 ? 0 : (q <= 4 ? q + 4 : q - 4); }

// D2V16 velocity set (Ark/Lib/D2V16.cpp:53-66): four rings of four directions, q = 4r + i,
// the opposite of q being 4r + (i + 2) mod 4.  The moments (Macro16, Ark/Lib/D2V16.cpp:125-145)
// odd in xi, and the entries of the inverse moment matrix (Ark/Lib/D2V16.cpp:14-52) that are
// not identically zero: the axis rings' rows (directions 0-3, 8-11) have none at the moments
// 1, 2, 4, 13 and, for the directions along x, 8, 10, 11 (along y: 7, 9, 12).  Row q' of the
// matrix holds row q's entries of the even moments and the negated entries of the odd ones.
__host__ __device__ constexpr int d2v16_opp(int q) { return (q & ~3) | ((q + 2) & 3); }
__host__ __device__ constexpr bool d2v16_odd_moment(int k) { return k == 1 || k == 2 || (k >= 7 && k <= 12); }
__host__ __device__ constexpr bool d2v16_entry(int j, int k) {
    return (j & 4) ? true
                   : !(k == 1 || k == 2 || k == 4 || k == 13 ||
                       ((j & 1) ? (k == 7 || k == 9 || k == 12) : (k == 8 || k == 10 || k == 11)));
}

// x * s for s in {-1, 0, 1}: exact, no multiply issued.
__device__ __forceinline__ double sx(int s, double x) { return s > 0 ? x : (s < 0 ? -x : 0.0); }

}  // namespace dugks
