// Case constants and device state of the FP32 deviation-storage path.
#pragma once
#include <cstddef>

// rest phase-field value the h deviations are taken from
#ifndef DUGKS_F32_PHI0
#define DUGKS_F32_PHI0 0.5
#endif
// |d phi/dx| below this is zero before grad(phi) is normalised (the reference's
// SetZero, Ark/Cpp/GradScheme.cpp:374-375, uses 1e-14 in FP64)
#ifndef DUGKS_F32_GCLAMP
#define DUGKS_F32_GCLAMP 1.0e-14
#endif

namespace dugks {
namespace f32 {

// Case constants of the fused deviation-form step in the storage type R
// (derived in FP64 on the host with the reference's expressions, then
// rounded once).  R = float is the FP32 storage path; R = double runs the
// same fused formulation in FP64.
template <typename R>
struct PR {
    int nx, ny, pitch, walls, model, gravity;
    int nee;  // NEE walls (Ark/Cpp/Boundary.cpp:140-184) instead of bounce-back
    int uw_grad;  // UW cell gradient: 0 6-point, 1 least squares, 2 4-point
    // slab partitions: global row of local row 0, and whether the rows below 0 /
    // from ny up are a neighbour's halo (2 rows of device memory) instead of a
    // wall or the periodic wrap; 0 for a whole grid
    int row0, halo_lo, halo_hi;
    R phi0, p0, aPhi, bPhi, Kp, RT, invRT, hDt, dt, Lambda0;
    R Beta, Kappa, PhiL, PhiV, RhoL, Gy;
    R inv_12dx, inv_12dy, inv_6dd, inv_wI_dphi, inv_RTdt;
    R tauf, aBP_f, ah_f;                       // flow relaxation after the first step
    R h_aBP, h_bBP, h_cBP, h_ah, h_bh, h_ch;  // phase-field relaxation
    R r_2dy, r_ndx, r_n2dx, r_ndy;             // reconstruction multipliers
    R aTP, bTP, dtV;
    R hneq;  // NEE: 2 TauMass / (2 TauMass + dt), the phase field's non-equilibrium factor
};
using P32 = PR<float>;

// init planes (first step only): the macroscopic state an initialisation left
enum { I_DPHI = 0, I_RHO, I_U, I_V, I_DP, I_TAU, I_SRCX, I_SRCY, I_RHOX, I_RHOY, I_FX, I_FY, I_N };
// aux planes: previous MacroSource outputs read by the next step
enum { A_FX = 0, A_FY, A_RHOX, A_RHOY, A_PPU, A_PPV, A_N };

// One copy of the state is PL_N planes [ny][pitch], one every qs elements:
//   f: the nine flow deviations f_q - f0_q;
//   g: the phase field's remainders g_q = h_q - w_q phi of the eight moving
//      directions q = 1..8 (h_0 follows from sum_q h_q = phi: g_0 = -sum g_q);
//   phi: the phase field itself as a float-float pair (head, tail);
//   aux: the previous MacroSource outputs.
// h_q - h0_q spans w_q/2 across an interface, and its FP32 rounding noise in phi (about
// 1e-8 per step) drove the velocity of a resting drop; the pair carries phi to ~1e-14
// and the remainders g_q are small, so what FP32 rounds is small.
constexpr int PL_F = 0, PL_G = 9, PL_PHI = 17, PL_AUX = 19, PL_N = PL_AUX + A_N;

// Scratch planes of the upwind (UW) step (fp32_uw.cu), one every qs floats:
//   B:   f-bar-plus pairs, 9 f planes then 9 h-relative (g) planes;
//   A:   the averaged-field inputs {srcx, srcy, rhox, rhoy, fx, fy};
//   INC: the collision increments B - T, laid out as B;
//   GX, GY: the 6-point gradients of the 18 B planes;  GP: the gradient of phi (x, y);
//   XF, YF: the six (f, h) flux pairs of each cell's west x-face / south y-face.
constexpr int UW_B = 0, UW_A = 18, UW_INC = 24, UW_GX = 42, UW_GY = 60, UW_GP = 78, UW_XF = 80, UW_YF = 92,
              UW_PLANES = 104;

template <typename R>
struct SR {
    R *df, *dg, *phi, *aux;      // the copy a step reads: planes PL_F, PL_G, PL_PHI, PL_AUX
    R *odf, *odg, *ophi, *oaux;  // the copy it writes (swapped with the above after each step)
    R *init;      // [I_N][ny][pitch]
    R *gphi;      // ghost phi rows [2 buffers][bottom, top][head, tail][pitch]
    size_t qs;    // plane stride (>= ny * pitch)
};
using S32 = SR<float>;

// the four plane groups of a copy that starts at base
template <typename R>
inline void set_copy(R *base, size_t qs, R *&f, R *&g, R *&phi, R *&aux) {
    f = base + PL_F * qs;
    g = base + PL_G * qs;
    phi = base + PL_PHI * qs;
    aux = base + PL_AUX * qs;
}

// Wall ghost rows of phi (the previous step's extrapolation 2 phi_0 - phi_1 below row 0
// and above row ny-1): phi as a float-float pair, head and tail rows.
constexpr int GPHI_ROWS = 8;
// first of the two rows (head, then tail) of buffer buf (0, 1) and side (0 bottom, 1 top)
__host__ __device__ __forceinline__ size_t gphi_row(int buf, int side) { return (size_t)(buf * 2 + side) * 2; }

// ---- FP32 storage of the pseudopotential models (D2Q9PP, D2V16)
// Constants: FP32 step coefficients, the velocity set, the rest equilibrium per
// unit density e_q = eq_q(1, 0, 0) (the state holds f_q - e_q rho), and the
// Carnahan-Starling constants in FP64 (the pressure and psi are evaluated from
// the FP64 density).
struct PPP {
    int nx, ny, pitch, model, Q;
    float hDt, dt, RT, invRT, Lambda0, Tau0, aTP, bTP, dtV;
    float r_2dy, r_ndx, r_n2dx, r_ndy, inv_6_2dx, inv_6_2dy;
    double R0, T_CS, aCS, RTd;
    // the same constants as float-float pairs (hi + lo) for the device arithmetic:
    // R0 T_CS, aCS, RT
    float rtcs_hi, rtcs_lo, acs_hi, acs_lo, rt_hi, rt_lo;
    float lat_hi, lat_lo;  // the lattice speed (velocities = lat times small integers) as hi + lo
    float xi_u[16], xi_v[16], w9[9], erest[16];
    // D2V16 inverse moment matrix of this case, by value: the kernels read its entries as
    // constant-bank operands (no loads), and cases of different lattice speed run side by
    // side with their own
    float iM16[16][16];
};
// One copy of the state the single-pass pseudopotential step reads or writes (two
// copies, swapped after each step: a strip segment reads rows its neighbours write)
struct PPV {
    float *g;                              // remainders [Q][ny][pitch]
    double *rho, *U, *V;                   // density and velocity
    float *psi, *psil, *scg;               // psi pair and its sign
    float *xFx, *xFy, *yFx, *yFy;          // face forces (read by the next step's face moments)
};

// State: the remainders g_q = f_q - e_q rho and the step's scratch in FP32, the
// density (and the pressure for output) in FP64; the density in two planes: the
// update reads its neighbours' density while it writes its own into rho_o, and the
// two swap after each step.
struct PPS {
    float *df, *bf;                  // g and the collision's remainders B_q - e_q rho [Q][ny][pitch]
    float *xb, *yb, *xfl, *yfl;      // face reconstructions and fluxes [Q][ny][pitch]
    float *xr, *yr, *xu, *yu, *xv, *yv, *xg, *yg, *xps, *yps;  // face rho, U, V, G, psi
    float *xFx, *xFy, *yFx, *yFy;    // face forces (kept for the next step's face velocity)
    double *rho, *rho_o, *p, *U, *V; // cell density (read / written by the update), pressure, velocity
    float *psi, *scg, *Fx, *Fy;
    float *psil, *xpsl, *ypsl;       // the tails of psi (cell, x faces, y faces) as float-float pairs
    PPV alt;                         // the single-pass step's second copy (its rho is rho_o)
    size_t qs;
};
// the copy of the state a step reads
inline PPV pp_current(const PPS &S) {
    return {S.df, S.rho, S.U, S.V, S.psi, S.psil, S.scg, S.xFx, S.xFy, S.yFx, S.yFy};
}
// after a single-pass step the written copy becomes the state
inline void pp_swap_copies(PPS &S) {
    PPV c = pp_current(S), a = S.alt;
    S.df = a.g, S.U = a.U, S.V = a.V, S.psi = a.psi, S.psil = a.psil, S.scg = a.scg;
    S.xFx = a.xFx, S.xFy = a.xFy, S.yFx = a.yFx, S.yFy = a.yFy;
    S.alt = c;
    S.alt.rho = nullptr;
}

// halo rows of a slab partition on each side
constexpr int SLAB_HALO = 2;

// cases one batched launch (serving) can hold: the size of the constant-memory case table
constexpr int BATCH_MAX_CASES = 64;

// after a step the written state becomes the one the next step reads
template <typename R>
inline void swap_io(SR<R> &S) {
    R *t = S.df; S.df = S.odf; S.odf = t;
    t = S.dg; S.dg = S.odg; S.odg = t;
    t = S.phi; S.phi = S.ophi; S.ophi = t;
    t = S.aux; S.aux = S.oaux; S.oaux = t;
}

}  // namespace f32
}  // namespace dugks
