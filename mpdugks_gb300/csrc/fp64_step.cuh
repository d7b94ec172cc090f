// FP64 DUGKS step kernels for sm_103a -- the plain drop-in path.
//
// One time step = three launches, in the phase order of
// Ark/Cpp/DUGKS2DSolver.cpp:175-327:
//   k_collide : [deferred P10 MacroSource of the previous step] + P1 + P2
//               (equilibria, force source, f-bar-plus; ghost phi rows)
//   k_faces   : P4 + P6 for every physical face (CD reconstruction, face
//               moments, face equilibrium/source, flux x xi.n dS, wall BB)
//   k_update  : P8 + P9 (finite-volume update, cell macros)
// The pseudopotential models split the face pass in two (face psi, then
// face force) -- the Jacobi semantics of the face psi gradient.
//
// This file is compiled twice (see fp64_exact.cu / fp64_fast.cu):
//  * DUGKS_EXACT = 1 with -fmad=false: every expression keeps the reference's
//    operand association, divisions stay divisions and nothing is contracted
//    into FMA, so the step reproduces the reference solver bit for bit (CUDA's
//    FP64 +, -, *, / and sqrt are correctly rounded, like the host's);
//  * DUGKS_EXACT = 0 with FMA contraction and reciprocal multiplies: the same
//    algorithm with fewer FP64 instructions, equal to the reference to rounding.
#pragma once
#include <cuda_runtime.h>
#include "dugks_device.cuh"

#ifndef DUGKS_EXACT
#error "define DUGKS_EXACT before including fp64_step.cuh"
#endif
#if DUGKS_EXACT
#define DUGKS_KNS exact
#define RDIV(x, d, invd) ((x) / (d))   // reference: a true division
// x / d with invd = RN(1/d), the reciprocal of a divisor shared by several quotients:
// correctly rounded (qdiv_rn), so the same double as the reference's division
#define QDIV(x, d, invd) qdiv_rn((x), (d), (invd))
#else
#define DUGKS_KNS fast
#define RDIV(x, d, invd) ((x) * (invd)) // one reciprocal, then multiplies
#define QDIV(x, d, invd) ((x) * (invd))
#endif

namespace dugks {
namespace DUGKS_KNS {


// x / d rounded to nearest, from y = RN(1/d): q0 = RN(x y) lies within an ulp of x / d,
// the residual r = x - d q0 is exact in one fused multiply-add, and RN(q0 + r y) is the
// correctly rounded quotient (P. Markstein, "Computation of elementary functions on the
// IBM RISC System/6000 processor", IBM J. Res. Develop. 34 (1990), Theorem 1; operands and
// quotient in the normal range).  Three FP64 operations where a division takes about ten;
// a zero x returns q0, which carries the quotient's sign.  Checked bit for bit against
// IEEE division on 2e8 random operand pairs (all-ones significands, near powers of two,
// signed zeros included).
__device__ __forceinline__ double qdiv_rn(double x, double d, double y) {
    const double q0 = __dmul_rn(x, y);
    const double r = __fma_rn(-d, q0, x);
    return x == 0.0 ? q0 : __fma_rn(r, y, q0);
}
__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
__device__ __forceinline__ void SetZero(double &d) { if (d < 1.0E-14 && d > -1.0E-14) d = 0.0; }  // Ark/Header/Mesh_2D.h:196-200

// Cell field at logical row j in -1..ny (ghost rows: 2 a0 - a1 with walls,
// wrap otherwise), column i already wrapped.
template <bool WALLS>
__device__ __forceinline__ double cellv(const double *__restrict__ a, int ny, int pitch, int j, int i) {
    if (j < 0) {
        if (WALLS) return 2.0 * a[i] - a[pitch + i];
        j += ny;
    } else if (j >= ny) {
        if (WALLS) return 2.0 * a[(size_t)(ny - 1) * pitch + i] - a[(size_t)(ny - 2) * pitch + i];
        j -= ny;
    }
    return a[(size_t)j * pitch + i];
}

// (xu*a + xv*b)/RT for the 9 D2Q9 directions from 4 divisions:
// a/RT, b/RT, (a+b)/RT, (b-a)/RT; the other directions are their negatives
// ((-x)/RT == -(x/RT) and -a + -b == -(a+b) exactly), direction 0 gives 0.
struct Xi4 {
    double a, b, s, d;
    __device__ __forceinline__ double get(int xu, int xv) const {
        if (xu == 0 && xv == 0) return 0.0;
        if (xv == 0) return xu > 0 ? a : -a;
        if (xu == 0) return xv > 0 ? b : -b;
        if (xu == xv) return xu > 0 ? s : -s;
        return xv > 0 ? d : -d;  // (-1,1): b - a;  (1,-1): a - b = -(b - a)
    }
};
__device__ __forceinline__ Xi4 xi4(double a, double b, double RT, double invRT) {
    (void)invRT;
    Xi4 r;
    r.a = QDIV(a, RT, invRT);
    r.b = QDIV(b, RT, invRT);
    r.s = QDIV(a + b, RT, invRT);
    r.d = QDIV(b - a, RT, invRT);
    return r;
}

// ---------------------------------------------------------------------------
// D2V16 equilibrium: Macro16 (Ark/Lib/D2V16.cpp:125-145) at T = T0, p = rho R0 T0,
// then the inverse moment matrix: row by row in the exact variant, by opposite pairs in
// the FMA variant, both without the structural zeros (the handle checks the matrix's form
// when it is made).
__device__ __forceinline__ void d2v16_eq(const Params &P, double rho, double u, double v, double *eq) {
    const double degrees = 3.0, degPlus2 = degrees + 2.0;
    const double T = P.T0, p = rho * P.R0 * T;
    const double u2 = u * u, v2 = v * v, RT = P.R0 * T;
    double M[16];
    M[0] = rho;
    M[1] = rho * u;
    M[2] = rho * v;
    M[3] = rho * (degrees * RT + u2 + v2);
    M[4] = M[1] * v;
    M[5] = rho * u2 + p;
    M[6] = rho * v2 + p;
    M[7] = M[1] * (degPlus2 * RT + u2 + v2);
    M[8] = M[2] * (degPlus2 * RT + u2 + v2);
    M[9] = M[1] * (3.0 * RT + u2);
    M[10] = M[2] * (3.0 * RT + v2);
    M[11] = M[2] * (RT + u2);
    M[12] = M[1] * (RT + v2);
    M[13] = ((degrees + 4.0) * RT + u2 + v2) * M[4];
    M[14] = degPlus2 * rho * RT * RT + p * ((degrees + 5.0) * u2 + v2) + rho * u2 * (u2 + v2);
    M[15] = degPlus2 * rho * RT * RT + p * ((degrees + 5.0) * v2 + u2) + rho * v2 * (u2 + v2);
#if DUGKS_EXACT
    // the reference's row sums in its order, less the terms of the matrix's structural zeros
    // (a sum that starts at +0 never becomes -0, so adding 0 * M[k] leaves it unchanged for
    // finite moments; a non-finite moment gives a non-finite sum either way), rows j and j'
    // together: the opposite row's product is t or -t exactly, (-a) m = -(a m)
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const int jo = d2v16_opp(j);
        if (jo < j) continue;
        double s = 0, so = 0;
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            if (!d2v16_entry(j, k)) continue;
            const double t = __ldg(P.iM16 + j * 16 + k) * M[k];
            s += t;
            so += d2v16_odd_moment(k) ? -t : t;
        }
        eq[j] = s;
        eq[jo] = so;
    }
#else
    // per opposite pair the even and odd partial sums over the matrix entries that are not
    // identically zero (d2v16_entry, d2v16_odd_moment): eq_j = E + O, eq_j' = E - O; 100
    // multiply-adds and loads instead of 256
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const int jo = d2v16_opp(j);
        if (jo < j) continue;
        double E = 0, O = 0;
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            if (!d2v16_entry(j, k)) continue;
            if (d2v16_odd_moment(k)) O += __ldg(P.iM16 + j * 16 + k) * M[k];
            else E += __ldg(P.iM16 + j * 16 + k) * M[k];
        }
        eq[j] = E + O;
        eq[jo] = E - O;
    }
#endif
}

// D2Q9PP equilibrium (Ark/Lib/D2Q9PP.cpp:51-62).
__device__ __forceinline__ void d2q9pp_eq(const Params &P, double rho, double U, double V, double *eq) {
    const double uu = U * U + V * V;
    const double invRT = P.r_RT;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const int xu = d2q9_xu(q), xv = d2q9_xv(q);
        double u1 = QDIV(sx(xu, U) + sx(xv, V), P.RT, invRT);
        eq[q] = d2q9_w(q) * rho * (1.0 + u1 + 0.5 * u1 * u1 - uu * P.Lambda0);
    }
}

template <int MODEL>
__device__ __forceinline__ void pp_eq(const Params &P, double rho, double U, double V, double *eq) {
    if (MODEL == PP16) d2v16_eq(P, rho, U, V, eq);
    else d2q9pp_eq(P, rho, U, V, eq);
}

#if !DUGKS_EXACT
// FMA variant: the He-Shan-Doolen projections (xi_q - u).F by opposite pairs, d - w and
// -d - w with d = xi_q.F, w = u.F (xi_q' = -xi_q); a rest direction has -w.  The exact
// variant keeps the reference's fx (xi_u - U) + fy (xi_v - V).
template <int MODEL>
__device__ __forceinline__ void pp_src_proj(const Params &P, double fx, double fy, double U, double V, double *pr) {
    constexpr int Q = MODEL == PP16 ? 16 : 9;
    const double w = fx * U + fy * V;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int qo = MODEL == PP16 ? d2v16_opp(q) : d2q9_bb(q);
        if (qo < q) continue;
        if (qo == q) {
            pr[q] = -w;
            continue;
        }
        const double d = fx * P.xi_u[q] + fy * P.xi_v[q];
        pr[q] = d - w;
        pr[qo] = -d - w;
    }
}
#endif

// Carnahan-Starling, b = 4 (Ark/Lib/nonidealEoS.h:114-118) and calcPsi
// (Ark/Header/Macroscopic.h:64-68).
__device__ __forceinline__ double cs_pressure(const Params &P, double rho) {
    return rho * P.R0 * P.T_CS * (1.0 + rho + rho * rho - rho * rho * rho) /
               ((1.0 - rho) * (1.0 - rho) * (1.0 - rho)) -
           P.aCS * rho * rho;
}
__device__ __forceinline__ void calc_psi(const Params &P, double rho, double p, double &scg, double &psi) {
    double G = (double)((p > rho * P.RT) - (p < rho * P.RT));
    scg = G;
    psi = sqrt(2 * (p - rho * P.RT) / G);
}

// 8-neighbour isotropic gradient (Ark/Lib/GradSchemeBasic.h:153-208).
// r: RN(1/(d2 6)) (Params r_g6x / r_g6y)
__device__ __forceinline__ double iso_gx(double E, double W, double NE, double NW, double SE, double SW, double d2,
                                         double r) {
    return QDIV(4 * (E - W) + 1 * (NE - NW + SE - SW), d2 * 6, r);
}
__device__ __forceinline__ double iso_gy(double N, double S, double NE, double NW, double SE, double SW, double d2,
                                         double r) {
    return QDIV(4 * (N - S) + 1 * (NE - SE + NW - SW), d2 * 6, r);
}

// ---------------------------------------------------------------------------
// MacroSource (Ark/Cpp/SourceM.cpp:35-62) with Grad_Phi_6points
// (Ark/Cpp/GradScheme.cpp:347-376).  Ghost phi rows come from the P2
// extrapolation of the step that produced phi (gphi buffer `gin`).
template <bool WALLS>
__device__ __forceinline__ void macro_source(const Params &P, const State &S, int i, int j, int gin, double phi,
                                             double rho, double U, double V, double ppu_old, double ppv_old,
                                             double &srcx, double &srcy, double &rhox, double &rhoy, double &fx,
                                             double &fy) {
    const int nx = P.nx, ny = P.ny, pitch = P.pitch;
    const double *__restrict__ PH = S.fld[F_PHI];
    const int im = wrapi(i - 1, nx), ip = wrapi(i + 1, nx);
    auto at = [&](int jj, int ii) -> double {
        if (jj < 0) return WALLS ? S.gphi[(size_t)(gin * 2 + 0) * pitch + ii] : PH[(size_t)(ny - 1) * pitch + ii];
        if (jj >= ny) return WALLS ? S.gphi[(size_t)(gin * 2 + 1) * pitch + ii] : PH[ii];
        return PH[(size_t)jj * pitch + ii];
    };
    const double E = at(j, ip), W = at(j, im), N = at(j + 1, i), Sd = at(j - 1, i);
    const double NE = at(j + 1, ip), NW = at(j + 1, im), SW = at(j - 1, im), SE = at(j - 1, ip);
    double Phi_x = iso_gx(E, W, NE, NW, SE, SW, P._2dx, P.r_g6x);
    double Phi_y = iso_gy(N, Sd, NE, NW, SE, SW, P._2dy, P.r_g6y);
    const double lap = QDIV(4 * (E + N + W + Sd) + (NE + NW + SW + SE) - 20 * phi, 6 * P.MinL * P.MinL, P.r_lap);
    SetZero(Phi_x);
    SetZero(Phi_y);
    const double F = 2 * P.Beta * (phi - P.PhiL) * (phi - P.PhiV) * (2 * phi - P.PhiL - P.PhiV) - P.Kappa * lap;
    rhox = P.aPhi * Phi_x;
    rhoy = P.aPhi * Phi_y;
    fx = F * Phi_x;
    fy = F * Phi_y;
    if (P.gravity) fy -= P.Gy * (rho - P.RhoL);
    const double L = sqrt(Phi_x * Phi_x + Phi_y * Phi_y);
    const double dU = phi * U - ppu_old, dV = phi * V - ppv_old;
    if (L != 0) {
        const double tmp = QDIV(-4 * (phi - P.PhiL) * (phi - P.PhiV), P.wI * (P.PhiL - P.PhiV), P.r_wI);
        const double rL = 1.0 / L;
        srcx = QDIV(Phi_x * tmp, L, rL) + QDIV(dU, P.RT * P.dt, P.r_RTdt);
        srcy = QDIV(Phi_y * tmp, L, rL) + QDIV(dV, P.RT * P.dt, P.r_RTdt);
    } else {
        srcx = QDIV(dU, P.RT * P.dt, P.r_RTdt);
        srcy = QDIV(dV, P.RT * P.dt, P.r_RTdt);
    }
}

// ---------------------------------------------------------------------------
// Collision pre-step.  MODEL AC/HCZ: Update_phi_Eq + Update_DVDF_Source +
// Update_phi_BP (Ark/Lib/D2Q9AC.cpp:69-105,331-344, Ark/Lib/D2Q9HCZ.cpp:54-92,
// Ark/Cpp/DUGKS2DSolver.cpp:379-401); PP: Ark/Lib/D2Q9PP.cpp:51-62,137-145.
// do_msrc: run the previous step's MacroSource / pseudopotential cell force
// (Ark/Cpp/PseudoP.cpp:31-38) first.
template <int MODEL, bool WALLS>
__global__ void __launch_bounds__(256) k_collide(Params P, State S, int do_msrc, int gin, int gout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= P.nx || j >= P.ny) return;
    const int pitch = P.pitch;
    const size_t c = (size_t)j * pitch + i;
    const double rho = S.fld[F_RHO][c], U = S.fld[F_U][c], V = S.fld[F_V][c], tau = S.fld[F_TAU][c];
    const double aBP = (2.0 * tau - P.hDt) / (2.0 * tau + P.dt), bBP = 1.0 - aBP, cBP = tau * bBP;
    if (MODEL == AC || MODEL == HCZ) {
        const double phi = S.fld[F_PHI][c], p = S.fld[F_P][c];
        double srcx, srcy, rhox, rhoy, fx, fy;
        if (do_msrc) {
            const double ppu = S.fld[F_PPU][c], ppv = S.fld[F_PPV][c];
            macro_source<WALLS>(P, S, i, j, gin, phi, rho, U, V, ppu, ppv, srcx, srcy, rhox, rhoy, fx, fy);
            S.fld[F_PHIX][c] = srcx;
            S.fld[F_PHIY][c] = srcy;
            S.fld[F_RHOX][c] = rhox;
            S.fld[F_RHOY][c] = rhoy;
            S.fld[F_FX][c] = fx;
            S.fld[F_FY][c] = fy;
            S.fld[F_PPU][c] = phi * U;
            S.fld[F_PPV][c] = phi * V;
        } else {
            srcx = S.fld[F_PHIX][c];
            srcy = S.fld[F_PHIY][c];
            rhox = S.fld[F_RHOX][c];
            rhoy = S.fld[F_RHOY][c];
            fx = S.fld[F_FX][c];
            fy = S.fld[F_FY][c];
        }
        if (WALLS) {  // P2: ghost phi for the next MacroSource (Ark/Cpp/Boundary.cpp:38-63)
            if (j == 0) S.gphi[(size_t)(gout * 2 + 0) * pitch + i] = 2.0 * phi - S.fld[F_PHI][c + pitch];
            if (j == P.ny - 1) S.gphi[(size_t)(gout * 2 + 1) * pitch + i] = 2.0 * phi - S.fld[F_PHI][c - pitch];
        }
        const double invRT = P.r_RT;
        const double pRT = QDIV(p, P.RT, invRT);
        const double uu = U * U + V * V;
        // (xi.a)/RT for xi in {0,+-1}^2 takes 4 distinct magnitudes; (-x)/RT == -(x/RT)
        Xi4 ur, fr;
        if (MODEL == AC) fr = xi4(fx, fy, P.RT, invRT);
        else ur = xi4(U, V, P.RT, invRT);
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const int xu = d2q9_xu(q), xv = d2q9_xv(q);
            const double w = d2q9_w(q);
            double hEq, fEq, fSo;
            if (MODEL == AC) {  // u = v = 0 (Ark/Lib/D2Q9AC.cpp:197-198): Gamma = 0, u1 = 0
                hEq = w * phi;
                fEq = w * pRT;
                if (q == 0) fEq -= pRT;
                fSo = w * fr.get(xu, xv);
            } else {
                const double u1 = ur.get(xu, xv);
                const double G = u1 + 0.5 * u1 * u1 - uu * P.Lambda0;
                const double cu = xu == 0 ? -U : (double)xu - U, cv = xv == 0 ? -V : (double)xv - V;  // 0 - U as -U
                hEq = w * (1.0 + u1) * phi;
                fEq = w * (p + rho * G * P.RT);
                fSo = w * ((1 + G) * (cu * fx + cv * fy) + G * P.RT * (cu * rhox + cv * rhoy));
            }
            const double hSo = (xu != 0 && xv != 0 ? sx(xu, srcx) + sx(xv, srcy)
                                                : (xu != 0 ? sx(xu, srcx) : sx(xv, srcy))) * w;
            const size_t o = (size_t)q * S.qs + c;
            if (WALLS && P.nee && (j == 0 || j == P.ny - 1)) {  // kept for the NEE wall faces
                const size_t wq = ((size_t)(j == 0 ? 0 : 1) * 9 + q) * pitch + i, ws = (size_t)2 * 9 * pitch;
                S.weq[wq] = fEq;
                S.weq[ws + wq] = fSo;
                S.weq[2 * ws + wq] = hEq;
                S.weq[3 * ws + wq] = hSo;
            }
            S.bh[o] = P.h_aBP * S.h[o] + P.h_bBP * hEq + P.h_cBP * hSo;
            S.bf[o] = aBP * S.f[o] + bBP * fEq + cBP * fSo;
        }
    } else {
        double fx, fy;
        if (do_msrc) {
            const int nx = P.nx, ny = P.ny;
            const int im = wrapi(i - 1, nx), ip = wrapi(i + 1, nx), jm = wrapi(j - 1, ny), jp = wrapi(j + 1, ny);
            const double *__restrict__ PS = S.fld[F_PSI];
            auto at = [&](int jj, int ii) { return PS[(size_t)jj * pitch + ii]; };
            const double gx = iso_gx(at(j, ip), at(j, im), at(jp, ip), at(jp, im), at(jm, ip), at(jm, im), P._2dx, P.r_g6x);
            const double gy = iso_gy(at(jp, i), at(jm, i), at(jp, ip), at(jp, im), at(jm, ip), at(jm, im), P._2dy, P.r_g6y);
            const double k = -S.fld[F_SCG][c] * at(j, i);
            fx = gx * k;
            fy = gy * k;
            S.fld[F_FX][c] = fx;
            S.fld[F_FY][c] = fy;
        } else {
            fx = S.fld[F_FX][c];
            fy = S.fld[F_FY][c];
        }
        constexpr int Q = MODEL == PP16 ? 16 : 9;
        double eq[Q];
        pp_eq<MODEL>(P, rho, U, V, eq);
        const double inv = 1.0 / (rho * P.RT);
#if !DUGKS_EXACT
        double pr[Q];
        pp_src_proj<MODEL>(P, fx, fy, U, V, pr);
#endif
#pragma unroll
        for (int q = 0; q < Q; ++q) {
#if DUGKS_EXACT
            const double So = QDIV((fx * (P.xi_u[q] - U) + fy * (P.xi_v[q] - V)) * eq[q], rho * P.RT, inv);
#else
            const double So = pr[q] * eq[q] * inv;
#endif
            const size_t o = (size_t)q * S.qs + c;
            S.bf[o] = aBP * S.f[o] + bBP * eq[q] + cBP * So;
        }
    }
}

// ---------------------------------------------------------------------------
// Face reconstruction CD_Interior_phi_Bh (Ark/Cpp/DUGKS2DSolver.cpp:604-687)
// for velocity q of one face.  XF: x-face between L=(im,j) and R=(i,j);
// else y-face between B=(i,j-1) and T=(i,j).
template <bool XF, bool WALLS>
__device__ __forceinline__ double face_bh(const Params &P, const double *__restrict__ B, int i, int im, int ip,
                                          int j, double xu, double xv) {
    const int ny = P.ny, pitch = P.pitch;
    // Denominators: the reference divides by _dx = xo - xn = -dx (normal) and by
    // 2(x1 - x0) = +-2d (tangential).  When dx, dy are powers of two (grad_mul)
    // the division is the exact multiply by the reciprocal, and
    // 0.5a + 0.5b == 0.5(a + b) exactly (power-of-two scaling commutes with
    // rounding away from the subnormal range), so these forms round alike.
    double o, n, gx, gy;
    if (XF) {
        o = cellv<WALLS>(B, ny, pitch, j, im);
        n = cellv<WALLS>(B, ny, pitch, j, i);
        const double SL = cellv<WALLS>(B, ny, pitch, j - 1, im), SR = cellv<WALLS>(B, ny, pitch, j - 1, i);
        const double NL = cellv<WALLS>(B, ny, pitch, j + 1, im), NR = cellv<WALLS>(B, ny, pitch, j + 1, i);
        if (P.grad_mul) {
            gy = (0.5 * ((NR - SR) + (NL - SL))) * P.r_2dy;
            gx = (o - n) * P.r_ndx;
        } else {
            gy = (0.5 * (NR - SR) + 0.5 * (NL - SL)) / (2 * P.dy);
            gx = (o - n) / (-P.dx);
        }
    } else {
        o = cellv<WALLS>(B, ny, pitch, j - 1, i);
        n = cellv<WALLS>(B, ny, pitch, j, i);
        const double WB = cellv<WALLS>(B, ny, pitch, j - 1, im), EB = cellv<WALLS>(B, ny, pitch, j - 1, ip);
        const double WT = cellv<WALLS>(B, ny, pitch, j, im), ET = cellv<WALLS>(B, ny, pitch, j, ip);
        if (P.grad_mul) {
            gx = (0.5 * ((WT - ET) + (WB - EB))) * P.r_n2dx;
            gy = (o - n) * P.r_ndy;
        } else {
            gx = (0.5 * (WT - ET) + 0.5 * (WB - EB)) / (2 * (-P.dx));
            gy = (o - n) / (-P.dy);
        }
    }
    return 0.5 * (o + n) - P.hDt * (gx * xu + gy * xv);
}

// The same for a D2Q9 velocity xi = (xu, xv), components in {-1, 0, 1} known at compile
// time after unrolling: a gradient a zero component multiplies is not formed (the
// product with 0 and its sum with the other term only decide the sign of a zero
// result), and a product with +-1 is the operand or its negation (exact); the
// nonzero terms keep the reference's order and rounding.
template <bool XF, bool WALLS>
__device__ __forceinline__ double face_bh9(const Params &P, const double *__restrict__ B, int i, int im, int ip,
                                           int j, int xu, int xv) {
    const int ny = P.ny, pitch = P.pitch;
    double o, n, gx = 0.0, gy = 0.0;
    if (XF) {
        o = cellv<WALLS>(B, ny, pitch, j, im);
        n = cellv<WALLS>(B, ny, pitch, j, i);
        if (xv != 0) {
            const double SL = cellv<WALLS>(B, ny, pitch, j - 1, im), SR = cellv<WALLS>(B, ny, pitch, j - 1, i);
            const double NL = cellv<WALLS>(B, ny, pitch, j + 1, im), NR = cellv<WALLS>(B, ny, pitch, j + 1, i);
            gy = P.grad_mul ? (0.5 * ((NR - SR) + (NL - SL))) * P.r_2dy
                            : (0.5 * (NR - SR) + 0.5 * (NL - SL)) / (2 * P.dy);
        }
        if (xu != 0) gx = P.grad_mul ? (o - n) * P.r_ndx : (o - n) / (-P.dx);
    } else {
        o = cellv<WALLS>(B, ny, pitch, j - 1, i);
        n = cellv<WALLS>(B, ny, pitch, j, i);
        if (xu != 0) {
            const double WB = cellv<WALLS>(B, ny, pitch, j - 1, im), EB = cellv<WALLS>(B, ny, pitch, j - 1, ip);
            const double WT = cellv<WALLS>(B, ny, pitch, j, im), ET = cellv<WALLS>(B, ny, pitch, j, ip);
            gx = P.grad_mul ? (0.5 * ((WT - ET) + (WB - EB))) * P.r_n2dx
                            : (0.5 * (WT - ET) + 0.5 * (WB - EB)) / (2 * (-P.dx));
        }
        if (xv != 0) gy = P.grad_mul ? (o - n) * P.r_ndy : (o - n) / (-P.dy);
    }
    const double avg = 0.5 * (o + n);
    if (xu == 0 && xv == 0) return avg;
    double g;
    if (xu != 0 && xv != 0) g = sx(xu, gx) + sx(xv, gy);
    else if (xu != 0) g = sx(xu, gx);
    else g = sx(xv, gy);
    return avg - P.hDt * g;
}

// ---------------------------------------------------------------------------
// UW flux scheme (_FLUX_SCHEME_UW_ARK), periodic grids.
//
// Cell gradients of f-bar-plus, Grad_VS_6points (Ark/Cpp/GradScheme.cpp:205-218,
// Ark/Lib/GradSchemeBasic.h:95-126): apsi = 4 on the axis neighbours, bpsi = 1
// on the diagonals (C0..C3 = E, N, W, S; D0..D3 = NE, NW, SW, SE), divided by
// 6 _2dx, in the reference's operand order.
template <int MODEL>
__global__ void __launch_bounds__(256) k_grad6(Params P, State S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= P.nx || j >= P.ny) return;
    const int pitch = P.pitch;
    const int im = wrapi(i - 1, P.nx), ip = wrapi(i + 1, P.nx), jm = wrapi(j - 1, P.ny), jp = wrapi(j + 1, P.ny);
    const size_t c = (size_t)j * pitch + i;
    const size_t cE = (size_t)j * pitch + ip, cW = (size_t)j * pitch + im, cN = (size_t)jp * pitch + i,
                 cS = (size_t)jm * pitch + i, cNE = (size_t)jp * pitch + ip, cNW = (size_t)jp * pitch + im,
                 cSW = (size_t)jm * pitch + im, cSE = (size_t)jm * pitch + ip;
    const double dxd = P._2dx * 6, dyd = P._2dy * 6, rdx = 1.0 / dxd, rdy = 1.0 / dyd;
    (void)rdx;
    (void)rdy;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
#pragma unroll
        for (int w = 0; w < 2; ++w) {
            const double *B = (w ? S.bh : S.bf) + (size_t)q * S.qs;
            const double E = B[cE], W = B[cW], N = B[cN], Sv = B[cS];
            double gx, gy;
            if (P.uw_grad == 1) {
                // Grad_VS_LS (Ark/Lib/GradSchemeBasic.h:127-152): sum over the neighbours
                // E, N, W, S of w_k (B_k - B_c), then the inverse 2x2 matrix.  On this
                // mesh of unit cells the weights of Grad_LSMatrix (:13-75) are exact: the
                // cell centres (two-triangle centroids, Ark/Cpp/Mesh/Cell_2D.cpp:157-179)
                // are i + 1/2, j + 1/2 and the periodic shadows' are offset by exactly
                // Lx / Ly, so wdx = {1, 0, -1, 0}, wdy = {0, 1, 0, -1} and the inverse
                // matrix is {{0.5, -0}, {-0, 0.5}}; every product and sum of the reference
                // is kept (the zero terms included), so the result is the same bits.
                const double C = B[c];
                const double nb[4] = {E, N, W, Sv}, wx[4] = {1.0, 0.0, -1.0, 0.0}, wy[4] = {0.0, 1.0, 0.0, -1.0};
                double sx = 0.0, sy = 0.0;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    sx = sx + wx[k] * (nb[k] - C);
                    sy = sy + wy[k] * (nb[k] - C);
                }
                gx = 0.5 * sx + -0.0 * sy;
                gy = -0.0 * sx + 0.5 * sy;
            } else if (P.uw_grad == 2) {
                // Grad_VS_4points (Ark/Lib/GradSchemeBasic.h:76-94): (C0 - C2) / (2 dx)
                gx = QDIV(E - W, P._2dx, 0.5 / P.dx);
                gy = QDIV(N - Sv, P._2dy, 0.5 / P.dy);
            } else {
                const double NE = B[cNE], NW = B[cNW], SW = B[cSW], SE = B[cSE];
                gx = QDIV(4.0 * (E - W) + (((NE - NW) + SE) - SW), dxd, rdx);
                gy = QDIV(4.0 * (N - Sv) + (((NE - SE) + NW) - SW), dyd, rdy);
            }
            (w ? S.ghx : S.gfx)[(size_t)q * S.qs + c] = gx;
            (w ? S.ghy : S.gfy)[(size_t)q * S.qs + c] = gy;
        }
    }
}

// Reconstruction UW_Interior_phi_Bh (Ark/Cpp/DUGKS2DSolver.cpp:558-603, chosen by the
// sign of xi.n dS at :689-706) of velocity (xu, xv) at one face: the upwind
// cell's f-bar-plus + (dx gx + dy gy) with (dx, dy) = x_f - hDt xi - x_c; the
// owner's and the neighbour's values averaged (owner first) along the face.
// The face is at the origin and its two cells at -1/2 ("o", below / left) and
// +1/2 ("n") along the normal: every offset is exact, as the reference's are
// on the unit grid.  The reference computes a periodic boundary face twice, as
// the high-side face (owner o, normal +x / +y: the interior form) and as the
// low-side face (owner n inside the domain, normal -x / -y): lo selects that form.
template <bool XF>
__device__ __forceinline__ double face_uw(const Params &P, const double *__restrict__ B,
                                          const double *__restrict__ GX, const double *__restrict__ GY, size_t co,
                                          size_t cn, double xu, double xv, bool lo) {
    const double xon = XF ? -0.5 : 0.0, yon = XF ? 0.0 : -0.5;  // centre of o
    const double xnn = XF ? 0.5 : 0.0, ynn = XF ? 0.0 : 0.5;    // centre of n
    const double xsh = 0.0 - P.hDt * xu, ysh = 0.0 - P.hDt * xv;
    const double dxo = xsh - xon, dyo = ysh - yon, dxn = xsh - xnn, dyn = ysh - ynn;
    const double Xo = dxo * GX[co] + dyo * GY[co], Xn = dxn * GX[cn] + dyn * GY[cn];
    const double xin = XF ? xu : xv;
    const double s = lo ? -xin : xin;  // xi.n of the reference's face
    if (lo) {                          // owner n, neighbour o
        if (s > 0) return B[cn] + Xn;
        if (s < 0) return B[co] + Xo;
        double t = B[cn] + Xn;
        t = t + B[co];
        t = t + Xo;
        return t / 2;
    }
    if (s > 0) return B[co] + Xo;
    if (s < 0) return B[cn] + Xn;
    double t = B[co] + Xo;
    t = t + B[cn];
    t = t + Xn;
    return t / 2;
}

// Allen-Cahn face: Update_MacroVar_h + Update_phi_Eqh + Update_DVDF_Source_h
// + Update_phi_h + Update_phiFlux_h (+ Wall_3_BB) -- Ark/Lib/D2Q9AC.cpp:106-144,
// 232-329,345-358; Ark/Lib/D2Q9HCZ.cpp:93-131,183-271;
// Ark/Cpp/DUGKS2DSolver.cpp:402-441; Ark/Cpp/Boundary.cpp:118-139.
// UW: blockIdx.z 2 and 3 are the x and y periodic boundary faces in the
// reference's low-side form (column 0 / row 0 only), written to xlo / ylo.
template <int MODEL, bool WALLS, bool UW>
__global__ void __launch_bounds__(256) k_faces_ac(Params P, State S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool xf = (blockIdx.z & 1) == 0;
    const bool lo = UW && blockIdx.z >= 2;
    const int nrows = xf ? P.ny : (WALLS ? P.ny + 1 : P.ny);
    if (i >= P.nx || j >= nrows) return;
    if (lo && (xf ? i != 0 : j != 0)) return;
    const int nx = P.nx, ny = P.ny, pitch = P.pitch;
    const int im = wrapi(i - 1, nx), ip = wrapi(i + 1, nx);
    // owner/neighbour cells of this face and the averaged source fields
    int jo, io;
    if (xf) { jo = j; io = im; } else { jo = j - 1; io = i; }
    if (UW && jo < 0) jo += ny;  // periodic y (UW runs without walls)
    double avg[6];
    const int fid[6] = {F_PHIX, F_PHIY, F_RHOX, F_RHOY, F_FX, F_FY};
#pragma unroll
    for (int k = 0; k < 6; ++k)
        avg[k] = 0.5 * (cellv<WALLS>(S.fld[fid[k]], ny, pitch, jo, io) + cellv<WALLS>(S.fld[fid[k]], ny, pitch, j, i));
    const double Phi_x = avg[0], Phi_y = avg[1], Rho_x = avg[2], Rho_y = avg[3], Fx = avg[4], Fy = avg[5];
    double bf[9], bh[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const double xu = d2q9_xu(q), xv = d2q9_xv(q);
        if (UW) {
            const size_t qo = (size_t)q * S.qs;
            const size_t co = (size_t)jo * pitch + io, cn = (size_t)j * pitch + i;
            if (xf) {
                bf[q] = face_uw<true>(P, S.bf + qo, S.gfx + qo, S.gfy + qo, co, cn, xu, xv, lo);
                bh[q] = face_uw<true>(P, S.bh + qo, S.ghx + qo, S.ghy + qo, co, cn, xu, xv, lo);
            } else {
                bf[q] = face_uw<false>(P, S.bf + qo, S.gfx + qo, S.gfy + qo, co, cn, xu, xv, lo);
                bh[q] = face_uw<false>(P, S.bh + qo, S.ghx + qo, S.ghy + qo, co, cn, xu, xv, lo);
            }
        } else if (xf) {
            bf[q] = face_bh9<true, WALLS>(P, S.bf + (size_t)q * S.qs, i, im, ip, j, d2q9_xu(q), d2q9_xv(q));
            bh[q] = face_bh9<true, WALLS>(P, S.bh + (size_t)q * S.qs, i, im, ip, j, d2q9_xu(q), d2q9_xv(q));
        } else {
            bf[q] = face_bh9<false, WALLS>(P, S.bf + (size_t)q * S.qs, i, im, ip, j, d2q9_xu(q), d2q9_xv(q));
            bh[q] = face_bh9<false, WALLS>(P, S.bh + (size_t)q * S.qs, i, im, ip, j, d2q9_xu(q), d2q9_xv(q));
        }
    }
    double Phi = 0, sumf = 0;
#pragma unroll
    for (int q = 0; q < 9; ++q) Phi += bh[q];
#pragma unroll
    for (int q = 0; q < 9; ++q) sumf += bf[q];
    const double Rho = P.aPhi * Phi + P.bPhi;
    const double invRT = P.r_RT;
    double U, V, p, Mu, tauh;
    if (MODEL == AC) {
        U = 0.0;
        V = 0.0;
        p = (sumf - bf[0]) * P.Kp;  // the u-dependent terms vanish with u = 0
        Mu = Rho * P.RT * P.Tau0;
        tauh = Mu / (Rho * P.RT);
    } else {
        // first moments over the directions with a nonzero component (the others add +-0)
        double su = 0, sv = 0;
#pragma unroll
        for (int q = 0; q < 9; ++q)
            if (d2q9_xu(q) != 0) su += sx(d2q9_xu(q), bf[q]);
#pragma unroll
        for (int q = 0; q < 9; ++q)
            if (d2q9_xv(q) != 0) sv += sx(d2q9_xv(q), bf[q]);
        const double inv = 1.0 / (Rho * P.RT);
        U = QDIV(su, Rho * P.RT, inv);
        V = QDIV(sv, Rho * P.RT, inv);
        U += QDIV(0.5 * P.hDt * Fx, Rho * P.RT, inv);
        V += QDIV(0.5 * P.hDt * Fy, Rho * P.RT, inv);
        p = sumf + 0.5 * P.hDt * P.RT * (Rho_x * U + Rho_y * V);
        Mu = P.NuV + (Phi - P.PhiV) * (P.NuL - P.NuV);
        Mu *= Rho;
        tauh = QDIV(Mu, Rho * P.RT, inv);
    }
    const double ah = 2.0 * tauh / (2.0 * tauh + P.hDt), bh_ = 1.0 - ah, ch = tauh * bh_;
    const double uu = U * U + V * V;
    const double pRT = QDIV(p, P.RT, invRT);
    Xi4 ur, fr;
    if (MODEL == AC) fr = xi4(Fx, Fy, P.RT, invRT);
    else ur = xi4(U, V, P.RT, invRT);
    double hf[9], hh[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const int xu = d2q9_xu(q), xv = d2q9_xv(q);
        const double w = d2q9_w(q);
        double hEq, fEq, fSo;
        if (MODEL == AC) {
            hEq = w * Phi;
            fEq = w * pRT;
            if (q == 0) fEq -= pRT;
            fSo = w * fr.get(xu, xv);
        } else {
            const double u1 = ur.get(xu, xv);
            const double G = u1 + 0.5 * u1 * u1 - uu * P.Lambda0;
            const double cu = xu == 0 ? -U : (double)xu - U, cv = xv == 0 ? -V : (double)xv - V;  // 0 - U as -U
            hEq = w * Phi * (1.0 + u1);
            fEq = w * (p + Rho * P.RT * G);
            fSo = w * ((1 + G) * (cu * Fx + cv * Fy) + G * P.RT * (cu * Rho_x + cv * Rho_y));
        }
        const double hSo = (xu != 0 && xv != 0 ? sx(xu, Phi_x) + sx(xv, Phi_y)
                                                : (xu != 0 ? sx(xu, Phi_x) : sx(xv, Phi_y))) * w;
        hh[q] = P.h_ah * bh[q] + P.h_bh * hEq + P.h_ch * hSo;
        hf[q] = ah * bf[q] + bh_ * fEq + ch * fSo;
    }
    if (WALLS && !xf && (j == 0 || j == ny)) {
        // bounce-back of the directions entering the fluid (xi.n_out < 0)
        const bool bottom = (j == 0);
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const int xv = d2q9_xv(q);
            if (bottom ? xv > 0 : xv < 0) {
                hh[q] = hh[d2q9_bb(q)];
                hf[q] = hf[d2q9_bb(q)];
            }
        }
    }
    double *outf = lo ? (xf ? S.xlo_f : S.ylo_f) : (xf ? S.xff : S.yff);
    double *outh = lo ? (xf ? S.xlo_h : S.ylo_h) : (xf ? S.xfh : S.yfh);
    const size_t qs = lo ? (xf ? (size_t)ny : (size_t)pitch) : (xf ? S.qs : S.qsy);
    const size_t c = lo ? (xf ? (size_t)j : (size_t)i) : (size_t)j * pitch + i;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const int s = xf ? d2q9_xu(q) : d2q9_xv(q);
        if (s == 0) continue;  // no flux along the face: the update does not read these slots
        outf[(size_t)q * qs + c] = sx(s, hf[q]);
        outh[(size_t)q * qs + c] = sx(s, hh[q]);
    }
}

// Wall_3_NEE (Ark/Cpp/Boundary.cpp:140-184) on the wall faces (y-face rows 0 and ny),
// written over what k_faces_ac left there.  The face's U, V keep the initial 0 of
// its MsQh (the routine never sets them); phi and rho are the owner's extrapolated
// with its Phi_x/Phi_y (the phase-field source vector after MacroSource) and
// Rho_x/Rho_y to the face (0.5 below / above the centre), p is the owner's;
// Update_phi_Eqh at those moments (Ark/Lib/D2Q9AC.cpp:106-144,
// Ark/Lib/D2Q9HCZ.cpp:93-131), plus the owner's non-equilibrium part
// (Tilde - Eq + hDt So, Eq and So of this step's collision) times
// 2 tau / (2 tau + dt); then Wall_3_BB.
template <int MODEL>
__global__ void __launch_bounds__(256) k_faces_nee(Params P, State S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, side = blockIdx.y;
    if (i >= P.nx) return;
    const int ny = P.ny, pitch = P.pitch, jc = side ? ny - 1 : 0;
    const size_t c = (size_t)jc * pitch + i;
    const double dxw = 0.0, dyw = side ? 0.5 : -0.5;
    const double Phi = S.fld[F_PHI][c] + S.fld[F_PHIX][c] * dxw + S.fld[F_PHIY][c] * dyw;
    const double Rho = S.fld[F_RHO][c] + S.fld[F_RHOX][c] * dxw + S.fld[F_RHOY][c] * dyw;
    const double p = S.fld[F_P][c], U = 0.0, V = 0.0;
    const double uu = U * U + V * V;
    const double tau = S.fld[F_TAU][c];
    const double hNEq = 2.0 * P.TauMass / (2.0 * P.TauMass + P.dt);
    const double fNEq = 2.0 * tau / (2.0 * tau + P.dt);
    const size_t ws = (size_t)2 * 9 * pitch;
    double hf[9], hh[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const double xu = d2q9_xu(q), xv = d2q9_xv(q), w = d2q9_w(q);
        const double u1 = (xu * U + xv * V) / P.RT;
        const double G = u1 + 0.5 * u1 * u1 - uu * P.Lambda0;
        const double hEq = w * Phi * (1.0 + u1);
        double fEq;
        if (MODEL == AC) {
            fEq = w * (p / P.RT + Rho * G);
            if (q == 0) fEq = fEq - 1.0 * p / P.RT;
        } else {
            fEq = w * (p + Rho * P.RT * G);
        }
        const size_t wq = ((size_t)side * 9 + q) * pitch + i, o = (size_t)q * S.qs + c;
        hh[q] = hEq + hNEq * (S.h[o] - S.weq[2 * ws + wq] + P.hDt * S.weq[3 * ws + wq]);
        hf[q] = fEq + fNEq * (S.f[o] - S.weq[wq] + P.hDt * S.weq[ws + wq]);
    }
    // bounce-back of the directions entering the fluid (xi.n_out < 0)
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const int xv = d2q9_xv(q);
        if (side ? xv < 0 : xv > 0) {
            hh[q] = hh[d2q9_bb(q)];
            hf[q] = hf[d2q9_bb(q)];
        }
    }
    const int jf = side ? ny : 0;
    const size_t cf = (size_t)jf * pitch + i;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const int xv = d2q9_xv(q);
        S.yff[(size_t)q * S.qsy + cf] = sx(xv, hf[q]);
        S.yfh[(size_t)q * S.qsy + cf] = sx(xv, hh[q]);
    }
}

// Pseudopotential face pass 1: BhDt, face moments with the previous face
// force, face pressure and psi (Ark/Lib/D2Q9PP.cpp:110-136, Ark/Cpp/PseudoP.cpp:23-30).
template <int MODEL>
__global__ void __launch_bounds__(256) k_faces_pp1(Params P, State S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool xf = blockIdx.z == 0;
    if (i >= P.nx || j >= P.ny) return;
    constexpr int Q = MODEL == PP16 ? 16 : 9;
    const int im = wrapi(i - 1, P.nx), ip = wrapi(i + 1, P.nx);
    const size_t c = (size_t)j * P.pitch + i;
    double R = 0, su = 0, sv = 0, b[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        b[q] = xf ? face_bh<true, false>(P, S.bf + (size_t)q * S.qs, i, im, ip, j, P.xi_u[q], P.xi_v[q])
                  : face_bh<false, false>(P, S.bf + (size_t)q * S.qs, i, im, ip, j, P.xi_u[q], P.xi_v[q]);
        (xf ? S.xbf : S.ybf)[(size_t)q * S.qs + c] = b[q];
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) R += b[q];
#pragma unroll
    for (int q = 0; q < Q; ++q) su += b[q] * P.xi_u[q];
#pragma unroll
    for (int q = 0; q < Q; ++q) sv += b[q] * P.xi_v[q];
    double U = su / R, V = sv / R;
    U += 0.5 * P.hDt * (xf ? S.xfFx : S.yfFx)[c] / R;
    V += 0.5 * P.hDt * (xf ? S.xfFy : S.yfFy)[c] / R;
    const double p = 1.0 * cs_pressure(P, R);
    double scg, psi;
    calc_psi(P, R, p, scg, psi);
    (xf ? S.xrho : S.yrho)[c] = R;
    (xf ? S.xu : S.yu)[c] = U;
    (xf ? S.xv : S.yv)[c] = V;
    (xf ? S.xscg : S.yscg)[c] = scg;
    (xf ? S.xpsi : S.ypsi)[c] = psi;
}

// Pseudopotential face pass 2: face force from the face-psi stencil
// (Ark/Cpp/PseudoP.cpp:39-46 over faceFaces, Ark/Lib/GradSchemeBasic.h:181-208),
// equilibrium, He-Shan-Doolen source and flux (Ark/Lib/D2Q9PP.cpp:97-105).
template <int MODEL>
__global__ void __launch_bounds__(256) k_faces_pp2(Params P, State S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool xf = blockIdx.z == 0;
    if (i >= P.nx || j >= P.ny) return;
    constexpr int Q = MODEL == PP16 ? 16 : 9;
    const int nx = P.nx, ny = P.ny, pitch = P.pitch;
    const int im = wrapi(i - 1, nx), ip = wrapi(i + 1, nx), jm = wrapi(j - 1, ny), jp = wrapi(j + 1, ny);
    const size_t c = (size_t)j * pitch + i;
    const double *__restrict__ PS = xf ? S.xpsi : S.ypsi;
    auto at = [&](int jj, int ii) { return PS[(size_t)jj * pitch + ii]; };
    const double gx = iso_gx(at(j, ip), at(j, im), at(jp, ip), at(jp, im), at(jm, ip), at(jm, im), P._2dx, P.r_g6x);
    const double gy = iso_gy(at(jp, i), at(jm, i), at(jp, ip), at(jp, im), at(jm, ip), at(jm, im), P._2dy, P.r_g6y);
    const double k = -(xf ? S.xscg : S.yscg)[c] * at(j, i);
    const double Fx = gx * k, Fy = gy * k;
    (xf ? S.xfFx : S.yfFx)[c] = Fx;
    (xf ? S.xfFy : S.yfFy)[c] = Fy;
    const double R = (xf ? S.xrho : S.yrho)[c], U = (xf ? S.xu : S.yu)[c], V = (xf ? S.xv : S.yv)[c];
    double eq[Q];
    pp_eq<MODEL>(P, R, U, V, eq);
    const double tauh = P.Tau0;
    const double ah = 2.0 * tauh / (2.0 * tauh + P.hDt), bh = 1.0 - ah, ch = tauh * bh;
    const double inv = 1.0 / (R * P.RT);
    const double *__restrict__ BB = xf ? S.xbf : S.ybf;
    double *out = xf ? S.xff : S.yff;
    const size_t qs = xf ? S.qs : S.qsy;
#if !DUGKS_EXACT
    double pr[Q];
    pp_src_proj<MODEL>(P, Fx, Fy, U, V, pr);
#endif
#pragma unroll
    for (int q = 0; q < Q; ++q) {
#if DUGKS_EXACT
        const double So = QDIV((Fx * (P.xi_u[q] - U) + Fy * (P.xi_v[q] - V)) * eq[q], R * P.RT, inv);
#else
        const double So = pr[q] * eq[q] * inv;
#endif
        const double t = ah * BB[(size_t)q * S.qs + c] + bh * eq[q] + ch * So;
        out[(size_t)q * qs + c] = t * (xf ? P.xi_u[q] : P.xi_v[q]);
    }
}

// ---------------------------------------------------------------------------
// Finite-volume update Update_phi_T (Ark/Cpp/DUGKS2DSolver.cpp:748-792) and
// cell macros Update_MacroVar (Ark/Lib/D2Q9AC.cpp:146-231,
// Ark/Lib/D2Q9HCZ.cpp:133-182, Ark/Lib/D2Q9PP.cpp:89-109).
template <int MODEL, bool WALLS>
__global__ void __launch_bounds__(256) k_update(Params P, State S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= P.nx || j >= P.ny) return;
    constexpr int Q = MODEL == PP16 ? 16 : 9;
    constexpr bool HASH = (MODEL == AC || MODEL == HCZ);
    const int pitch = P.pitch;
    const int ip = wrapi(i + 1, P.nx);
    const int jn = WALLS ? j + 1 : wrapi(j + 1, P.ny);
    const size_t c = (size_t)j * pitch + i;
    const size_t cE = (size_t)j * pitch + ip, cN = (size_t)jn * pitch + i;
    double sumf = 0, su = 0, sv = 0, Phi = 0, f0 = 0;
#pragma unroll
    // UW: the west face of column 0 and the south face of row 0 are the reference's
    // low-side periodic boundary faces (k_faces_ac, xlo / ylo)
    const bool xlo = P.uw && i == 0, ylo = P.uw && j == 0;
    for (int q = 0; q < Q; ++q) {
        const size_t oq = (size_t)q * S.qs, oy = (size_t)q * S.qsy;
        // net flux E, N, W, S in the reference's order.  D2Q9 Allen-Cahn: the faces
        // a direction runs along carry no flux (xi.n = 0: the reference adds exact zeros,
        // which only decide the sign of a zero sum; k_faces_ac does not store them), so
        // only the crossing faces are added and the rest direction has no flux term
        const bool cx = !HASH || d2q9_xu(q) != 0, cy = !HASH || d2q9_xv(q) != 0;
        double s = 0.0;
        if (cx && cy) {
            s = -S.xff[oq + cE];
            s += -S.yff[oy + cN];
            s += xlo ? S.xlo_f[(size_t)q * P.ny + j] : S.xff[oq + c];
            s += ylo ? S.ylo_f[(size_t)q * pitch + i] : S.yff[oy + c];
        } else if (cx) {
            s = -S.xff[oq + cE];
            s += xlo ? S.xlo_f[(size_t)q * P.ny + j] : S.xff[oq + c];
        } else if (cy) {
            s = -S.yff[oy + cN];
            s += ylo ? S.ylo_f[(size_t)q * pitch + i] : S.yff[oy + c];
        }
        const double fn = (cx || cy) ? P.aTP * S.bf[oq + c] - P.bTP * S.f[oq + c] + P.dtV * s
                                     : P.aTP * S.bf[oq + c] - P.bTP * S.f[oq + c];
        S.f[oq + c] = fn;
        sumf += fn;
        if (q == 0) f0 = fn;
        if (MODEL == PP16) {
            su += fn * P.xi_u[q];
            sv += fn * P.xi_v[q];
        } else {
            if (!HASH || d2q9_xu(q) != 0) su += sx(d2q9_xu(q), fn);
            if (!HASH || d2q9_xv(q) != 0) sv += sx(d2q9_xv(q), fn);
        }
        if (HASH) {
            double t = 0.0;
            if (cx && cy) {
                t = -S.xfh[oq + cE];
                t += -S.yfh[oy + cN];
                t += xlo ? S.xlo_h[(size_t)q * P.ny + j] : S.xfh[oq + c];
                t += ylo ? S.ylo_h[(size_t)q * pitch + i] : S.yfh[oy + c];
            } else if (cx) {
                t = -S.xfh[oq + cE];
                t += xlo ? S.xlo_h[(size_t)q * P.ny + j] : S.xfh[oq + c];
            } else if (cy) {
                t = -S.yfh[oy + cN];
                t += ylo ? S.ylo_h[(size_t)q * pitch + i] : S.yfh[oy + c];
            }
            const double hn = (cx || cy) ? P.aTP * S.bh[oq + c] - P.bTP * S.h[oq + c] + P.dtV * t
                                         : P.aTP * S.bh[oq + c] - P.bTP * S.h[oq + c];
            S.h[oq + c] = hn;
            Phi += hn;
        }
    }
    if (MODEL == AC || MODEL == HCZ) {
        const double Rho = P.aPhi * Phi + P.bPhi;
        double U, V, p, Mu, tau;
        if (MODEL == AC) {
            U = 0.0;
            V = 0.0;
            p = (sumf - f0) * P.Kp;  // (hDt rho_x.u - rho w0 |u|^2 lambda) vanishes with u = 0
            Mu = Rho * P.RT * P.Tau0;
            tau = Mu / (Rho * P.RT);
        } else {
            const double inv = 1.0 / (Rho * P.RT);
            U = QDIV(su, Rho * P.RT, inv);
            V = QDIV(sv, Rho * P.RT, inv);
            U += QDIV(P.hDt * S.fld[F_FX][c], Rho * P.RT, inv);
            V += QDIV(P.hDt * S.fld[F_FY][c], Rho * P.RT, inv);
            p = sumf + P.hDt * (S.fld[F_RHOX][c] * U + S.fld[F_RHOY][c] * V) * P.RT;
            Mu = P.NuV + (Phi - P.PhiV) * (P.NuL - P.NuV);
            Mu *= Rho;
            tau = QDIV(Mu, Rho * P.RT, inv);
        }
        S.fld[F_PHI][c] = Phi;
        S.fld[F_RHO][c] = Rho;
        S.fld[F_U][c] = U;
        S.fld[F_V][c] = V;
        S.fld[F_P][c] = p;
        S.fld[F_TAU][c] = tau;
    } else {
        const double Rho = sumf;
        const double invR = 1.0 / Rho;
        double U = QDIV(su, Rho, invR), V = QDIV(sv, Rho, invR);
        U += QDIV(P.hDt * S.fld[F_FX][c], Rho, invR);
        V += QDIV(P.hDt * S.fld[F_FY][c], Rho, invR);
        const double p = 1.0 * cs_pressure(P, Rho);
        double scg, psi;
        calc_psi(P, Rho, p, scg, psi);
        S.fld[F_RHO][c] = Rho;
        S.fld[F_U][c] = U;
        S.fld[F_V][c] = V;
        S.fld[F_P][c] = p;
        S.fld[F_SCG][c] = scg;
        S.fld[F_PSI][c] = psi;
    }
}

// Deferred MacroSource / pseudopotential cell force on its own (used before
// handing the fields to the host).
template <int MODEL, bool WALLS>
__global__ void __launch_bounds__(256) k_finalize(Params P, State S, int gin) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= P.nx || j >= P.ny) return;
    const size_t c = (size_t)j * P.pitch + i;
    if (MODEL == AC || MODEL == HCZ) {
        const double phi = S.fld[F_PHI][c], U = S.fld[F_U][c], V = S.fld[F_V][c];
        double srcx, srcy, rhox, rhoy, fx, fy;
        macro_source<WALLS>(P, S, i, j, gin, phi, S.fld[F_RHO][c], U, V, S.fld[F_PPU][c], S.fld[F_PPV][c], srcx,
                            srcy, rhox, rhoy, fx, fy);
        // neighbours read phi only, so in-place writes are race-free
        S.fld[F_PHIX][c] = srcx;
        S.fld[F_PHIY][c] = srcy;
        S.fld[F_RHOX][c] = rhox;
        S.fld[F_RHOY][c] = rhoy;
        S.fld[F_FX][c] = fx;
        S.fld[F_FY][c] = fy;
        S.fld[F_PPU][c] = phi * U;
        S.fld[F_PPV][c] = phi * V;
    } else {
        const int nx = P.nx, ny = P.ny, pitch = P.pitch;
        const int im = wrapi(i - 1, nx), ip = wrapi(i + 1, nx), jm = wrapi(j - 1, ny), jp = wrapi(j + 1, ny);
        const double *__restrict__ PS = S.fld[F_PSI];
        auto at = [&](int jj, int ii) { return PS[(size_t)jj * pitch + ii]; };
        const double gx = iso_gx(at(j, ip), at(j, im), at(jp, ip), at(jp, im), at(jm, ip), at(jm, im), P._2dx, P.r_g6x);
        const double gy = iso_gy(at(jp, i), at(jm, i), at(jp, ip), at(jp, im), at(jm, ip), at(jm, im), P._2dy, P.r_g6y);
        const double k = -S.fld[F_SCG][c] * at(j, i);
        S.fld[F_FX][c] = gx * k;
        S.fld[F_FY][c] = gy * k;
    }
}

// ---------------------------------------------------------------------------
// Reductions: per-block partial sums of rho, phi, (rho-rho_last)^2, rho^2,
// fixed-order tree (deterministic), then one block sums the partials.
__global__ void __launch_bounds__(256) k_reduce_partial(Params P, const double *__restrict__ rho,
                                                        const double *__restrict__ phi, double *rho_last,
                                                        double *partial, int has_phi) {
    __shared__ double sh[4][256];
    const int tid = threadIdx.x;
    const long n = (long)P.nx * P.ny;
    double a = 0, b = 0, d = 0, r2 = 0;
    for (long k = (long)blockIdx.x * blockDim.x + tid; k < n; k += (long)gridDim.x * blockDim.x) {
        const int j = (int)(k / P.nx), i = (int)(k % P.nx);
        const size_t c = (size_t)j * P.pitch + i;
        const double r = rho[c];
        a += r;
        if (has_phi) b += phi[c];
        const double dr = r - rho_last[c];
        d += dr * dr;
        r2 += r * r;
        rho_last[c] = r;
    }
    sh[0][tid] = a;
    sh[1][tid] = b;
    sh[2][tid] = d;
    sh[3][tid] = r2;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (tid < s)
            for (int m = 0; m < 4; ++m) sh[m][tid] += sh[m][tid + s];
        __syncthreads();
    }
    if (tid < 4) partial[(size_t)blockIdx.x * 4 + tid] = sh[tid][0];
}

__global__ void k_reduce_final(const double *__restrict__ partial, int nblocks, double *out) {
    __shared__ double sh[4][256];
    const int tid = threadIdx.x;
    double v[4] = {0, 0, 0, 0};
    for (int k = tid; k < nblocks; k += blockDim.x)
        for (int m = 0; m < 4; ++m) v[m] += partial[(size_t)k * 4 + m];
    for (int m = 0; m < 4; ++m) sh[m][tid] = v[m];
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (tid < s)
            for (int m = 0; m < 4; ++m) sh[m][tid] += sh[m][tid + s];
        __syncthreads();
    }
    if (tid < 4) out[tid] = sh[tid][0];
}

__global__ void k_check_finite(const double *__restrict__ a, size_t n, int *flag) {
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        if (!isfinite(a[k])) {
            atomicOr(flag, 1);
            return;
        }
}

// ---------------------------------------------------------------------------
// Host-side launch helpers (called from capi.cu).

template <int MODEL, bool WALLS>
static void launch_step_t(const Params &P, const State &S, int do_msrc, int gin, int gout, cudaStream_t st,
                          int64_t *launches, cudaEvent_t *ev) {
    const dim3 blk(32, 8);
    const dim3 grd((P.nx + 31) / 32, (P.ny + 7) / 8);
    if (ev) cudaEventRecord(ev[0], st);
    k_collide<MODEL, WALLS><<<grd, blk, 0, st>>>(P, S, do_msrc, gin, gout);
    if (ev) cudaEventRecord(ev[1], st);
    if constexpr (MODEL == AC || MODEL == HCZ) {
        if (!WALLS && P.uw) {  // UW: cell gradients, then the faces with the low-side boundary faces
            k_grad6<MODEL><<<grd, blk, 0, st>>>(P, S);
            const dim3 gf((P.nx + 31) / 32, (P.ny + 1 + 7) / 8, 4);
            k_faces_ac<MODEL, false, true><<<gf, blk, 0, st>>>(P, S);
            *launches += 4;
        } else {
            const dim3 gf((P.nx + 31) / 32, (P.ny + 1 + 7) / 8, 2);
            k_faces_ac<MODEL, WALLS, false><<<gf, blk, 0, st>>>(P, S);
            *launches += 3;
            if (WALLS && P.nee) {  // NEE wall faces over the bounce-back ones
                k_faces_nee<MODEL><<<dim3((P.nx + 127) / 128, 2), 128, 0, st>>>(P, S);
                *launches += 1;
            }
        }
    } else {
        const dim3 gf((P.nx + 31) / 32, (P.ny + 7) / 8, 2);
        k_faces_pp1<MODEL><<<gf, blk, 0, st>>>(P, S);
        k_faces_pp2<MODEL><<<gf, blk, 0, st>>>(P, S);
        *launches += 4;
    }
    if (ev) cudaEventRecord(ev[2], st);
    k_update<MODEL, WALLS><<<grd, blk, 0, st>>>(P, S);
    if (ev) cudaEventRecord(ev[3], st);
}

template <int MODEL, bool WALLS>
static void launch_finalize_t(const Params &P, const State &S, int gin, cudaStream_t st) {
    const dim3 blk(32, 8);
    const dim3 grd((P.nx + 31) / 32, (P.ny + 7) / 8);
    k_finalize<MODEL, WALLS><<<grd, blk, 0, st>>>(P, S, gin);
}

void launch_fp64_step(const Params &P, const State &S, int do_msrc, int gin, int gout, cudaStream_t st,
                      int64_t *launches, cudaEvent_t *ev) {
    switch (P.model * 2 + (P.walls ? 1 : 0)) {
        case AC * 2 + 0: launch_step_t<AC, false>(P, S, do_msrc, gin, gout, st, launches, ev); break;
        case AC * 2 + 1: launch_step_t<AC, true>(P, S, do_msrc, gin, gout, st, launches, ev); break;
        case HCZ * 2 + 0: launch_step_t<HCZ, false>(P, S, do_msrc, gin, gout, st, launches, ev); break;
        case HCZ * 2 + 1: launch_step_t<HCZ, true>(P, S, do_msrc, gin, gout, st, launches, ev); break;
        case PP9 * 2 + 0: launch_step_t<PP9, false>(P, S, do_msrc, gin, gout, st, launches, ev); break;
        case PP16 * 2 + 0: launch_step_t<PP16, false>(P, S, do_msrc, gin, gout, st, launches, ev); break;
        default: break;
    }
}

void launch_fp64_finalize(const Params &P, const State &S, int gin, cudaStream_t st, int64_t *launches) {
    switch (P.model * 2 + (P.walls ? 1 : 0)) {
        case AC * 2 + 0: launch_finalize_t<AC, false>(P, S, gin, st); break;
        case AC * 2 + 1: launch_finalize_t<AC, true>(P, S, gin, st); break;
        case HCZ * 2 + 0: launch_finalize_t<HCZ, false>(P, S, gin, st); break;
        case HCZ * 2 + 1: launch_finalize_t<HCZ, true>(P, S, gin, st); break;
        case PP9 * 2 + 0: launch_finalize_t<PP9, false>(P, S, gin, st); break;
        case PP16 * 2 + 0: launch_finalize_t<PP16, false>(P, S, gin, st); break;
        default: return;
    }
    *launches += 1;
}

void launch_reduce(const Params &P, const double *rho, const double *phi, double *rho_last, double *partial,
                   int nblocks, double *out4, int has_phi, cudaStream_t st, int64_t *launches) {
    k_reduce_partial<<<nblocks, 256, 0, st>>>(P, rho, phi, rho_last, partial, has_phi);
    k_reduce_final<<<1, 256, 0, st>>>(partial, nblocks, out4);
    *launches += 2;
}

void launch_check_finite(const double *a, size_t n, int *flag, cudaStream_t st, int64_t *launches) {
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    k_check_finite<<<blocks, 256, 0, st>>>(a, n, flag);
    *launches += 1;
}

}  // namespace DUGKS_KNS
}  // namespace dugks
