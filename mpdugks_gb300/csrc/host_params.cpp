// Host-side case setup: derived constants and initial states.
//
// derive_params evaluates the constant expressions of
// Ark/Constant/ZeroReference.h, Ark/Constant/ZeroNamespace.h, Ark/Lib/D2Q9.h,
// Ark/Lib/D2V16.h and Ark/Lib/nonidealEoS.h in the reference's order, so the
// device sees the same doubles the reference binary computes.
// host_init_state runs the reference initialisation functions' steps
// (Ark/Cpp/Preprocess.cpp) on the SoA layout.
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/dugks_gpu.h"
#include "dugks_device.cuh"

namespace dugks {

void derive_params(const dugks_case_t &cs, const dugks_grid_t &g, Params &P) {
    P = Params{};
    P.nx = g.nx;
    P.ny = g.ny;
    P.pitch = (g.nx + 31) / 32 * 32;
    P.walls = g.y_walls ? 1 : 0;
    P.model = cs.model;
    P.gravity = cs.Gy != 0.0 ? 1 : 0;
    const bool d2v16 = cs.model == DUGKS_MODEL_PP16;
    P.Q = d2v16 ? 16 : 9;
    // Ark/Constant/ZeroReference.h (ChLength = NL = Nx, X/Y from 0)
    const double ChLength = (double)g.nx;
    P.MinL = ChLength / g.nx;
    const double Lx = (double)g.nx - 0.0, Ly = (double)g.ny - 0.0;
    P.dx = Lx / g.nx;
    P.dy = Ly / g.ny;
    P.T0 = 1.0 / 3;
    P.R0 = 1.0;
    P.RT = P.R0 * P.T0;
    P.Lambda0 = 1 / (2.0 * P.R0 * P.T0);
    const double Rho0 = 1.0, Mu0 = cs.Mu0, Nu0 = Mu0 / Rho0;
    P.Tau0 = Nu0 / P.RT;
    // velocity model
    double MaxU, MaSpan;
    if (d2v16) {
        MaSpan = cs.d2v16_c;
        MaxU = 2 * MaSpan * std::sqrt(2.0);
    } else {
        MaxU = std::sqrt(3.0 * P.RT);
        MaSpan = std::sqrt(3.0 * P.RT);
    }
    P.c16 = MaSpan;
    // Ark/Constant/ZeroNamespace.h
    const double CFL = 0.5;
    P.dt = CFL > 0.0 ? CFL * P.MinL / MaxU : 1.0E-4;
    P.hDt = 0.5 * P.dt;
    const double Cn = cs.W / ChLength;
    P.wI = ChLength * Cn;
    P.Beta = 12.0 * cs.Sigma / P.wI;
    P.Kappa = 3.0 * cs.Sigma * P.wI / 2;
    P.PhiL = 1.0;
    P.PhiV = 0.0;
    P.RhoL = cs.RhoL;
    P.RhoV = cs.RhoV;
    P.NuL = Nu0;
    P.NuV = Nu0;
    P.aPhi = (P.RhoL - P.RhoV) / (P.PhiL - P.PhiV);
    P.bPhi = P.RhoV - P.aPhi * P.PhiV;
    P.Gy = cs.Gy;
    P.TauMass = cs.M_Phi / P.RT;
    P.Kp = P.RT * 9 / 5.0;        // Ark/Lib/D2Q9AC.cpp:32
    P._2dx = 2.0 * P.dx;          // Ark/Lib/GradSchemeBasic.h:7-11
    P._2dy = 2.0 * P.dy;
    P.aTP = 4.0 / 3.0;            // Ark/Cpp/DUGKS2DSolver.cpp:12
    P.bTP = 1.0 / 3.0;
    P.dtV = P.dt / (P.dx * P.dy); // DtSlashVolume, Ark/Cpp/Mesh/Cell_2D.cpp:182
    {   // constant phase-field relaxation (Cell_2D.cpp:120-125, Face_2D.cpp:306-311)
        const double tau = P.TauMass;
        P.h_aBP = (2.0 * tau - P.hDt) / (2.0 * tau + P.dt);
        P.h_bBP = 1.0 - P.h_aBP;
        P.h_cBP = tau * P.h_bBP;
        P.h_ah = 2.0 * tau / (2.0 * tau + P.hDt);
        P.h_bh = 1.0 - P.h_ah;
        P.h_ch = tau * P.h_bh;
    }
    {   // power-of-two spacings make every reconstruction division an exact multiply
        int e;
        const bool p2 = std::frexp(P.dx, &e) == 0.5 && std::frexp(P.dy, &e) == 0.5;
        P.grad_mul = p2 ? 1 : 0;
        P.r_ndx = 1.0 / (-P.dx);
        P.r_ndy = 1.0 / (-P.dy);
        P.r_2dy = 1.0 / (2 * P.dy);
        P.r_n2dx = 1.0 / (2 * (-P.dx));
    }
    {   // reciprocals of the divisors the device forms with the same expressions (IEEE
        // double here and there, so the same divisors and the same reciprocals)
        P.r_RT = 1.0 / P.RT;
        P.r_g6x = 1.0 / (P._2dx * 6);
        P.r_g6y = 1.0 / (P._2dy * 6);
        P.r_lap = 1.0 / (6 * P.MinL * P.MinL);
        P.r_wI = 1.0 / (P.wI * (P.PhiL - P.PhiV));
        P.r_RTdt = 1.0 / (P.RT * P.dt);
    }
    P.uw = cs.flux_scheme != DUGKS_FLUX_CD ? 1 : 0;
    P.uw_grad = cs.flux_scheme == DUGKS_FLUX_UW_LS ? 1 : (cs.flux_scheme == DUGKS_FLUX_UW_4P ? 2 : 0);
    P.nee = (cs.wall_scheme == DUGKS_WALL_NEE && g.y_walls) ? 1 : 0;
    P.T_CS = cs.Tr * cs.Tc_CS;
    P.aCS = cs.aCS;
    if (d2v16) {
        const double su[16] = {1, 0, -1, 0, 1, -1, -1, 1, 2, 0, -2, 0, 2, -2, -2, 2};
        const double sv[16] = {0, 1, 0, -1, 1, 1, -1, -1, 0, 2, 0, -2, 2, 2, -2, -2};
        for (int q = 0; q < 16; ++q) {
            P.xi_u[q] = su[q] * MaSpan;
            P.xi_v[q] = sv[q] * MaSpan;
            P.omega[q] = 0.0;
            P.bb[q] = q;
        }
    } else {
        for (int q = 0; q < 9; ++q) {
            P.xi_u[q] = MaSpan * d2q9_xu(q);
            P.xi_v[q] = MaSpan * d2q9_xv(q);
            P.omega[q] = d2q9_w(q);
            P.bb[q] = d2q9_bb(q);
        }
    }
}

// Inverse moment matrix of the D2V16 model, from the closed-form
// coefficients of Ark/Lib/D2V16.cpp:14-33 (c, e = (3+nK)c, nK = 0); the row
// and column layout is the reference's (Ark/Lib/D2V16.cpp:34-52).
void build_d2v16_matrix(double c, double out[16][16]) {
    const double e = 3.0 * c;
    const double c2 = c * c, e2 = e * e, c2e2 = c2 * e2;
    const double A = 1.0 / (4.0 * e2), B = (-21.0 * c2 - e2) / (48.0 * c2e2), D = (7.0 * c2 + e2) / (32.0 * c2e2),
                 E = (-3.0 * c2 - e2) / (96.0 * c2e2), F = 1.0 / (3.0 * c2),
                 G = (3.0 * c2 - 5.0 * e2) / (4.0 * e2 * (e2 - 3.0 * c2)),
                 H = 3.0 * (c2 + e2) / (4.0 * e2 * (e2 - 3.0 * c2)), I = (21.0 * c2 - 11.0 * e2) / (48.0 * c2e2),
                 J = (21.0 * c2 * c2 - 32.0 * c2e2 + 11.0 * e2 * e2) / (32.0 * c2e2 * (e2 - 3.0 * c2)),
                 K = (21.0 * c2 * c2 - 36.0 * c2e2 + 7.0 * e2 * e2) / (32.0 * c2e2 * (e2 - 3.0 * c2)),
                 L = (3.0 * c2 - 5.0 * e2) / (96.0 * c2e2), N = 1.0 / (2.0 * c * e2),
                 Pc = (3.0 * c2 - e2) / (12.0 * c2e2 * c), Qc = (c2 + e2) / (16.0 * c2e2 * c),
                 R = (c2 - e2) / (16.0 * c2e2 * c), S = 1.0 / (24.0 * c2 * c2), T = 1.0 / (4.0 * c2 * (e2 - 3.0 * c2)),
                 U = (c2 - e2) / (32.0 * c2 * c2 * (e2 - 3.0 * c2)),
                 V = (5.0 * c2 - e2) / (32.0 * c2 * c2 * (e2 - 3.0 * c2));
    // rows: ring 1 (axis c), ring 2 (diagonal c), ring 3 (axis 2c), ring 4 (diagonal 2c)
    const double ic = 1.0 / (3.0 * c), jc = 1.0 / (24 * c);
    const double m[16][16] = {
        {0, 0, 0, A, 0, G, H, N, 0, -N, 0, 0, -N, 0, T, -T},
        {0, 0, 0, A, 0, H, G, 0, N, 0, -N, -N, 0, 0, -T, T},
        {0, 0, 0, A, 0, G, H, -N, 0, N, 0, 0, N, 0, T, -T},
        {0, 0, 0, A, 0, H, G, 0, -N, 0, N, N, 0, 0, -T, T},
        {2.0 / 3.0, ic, ic, B, F, I, I, -N / 2, -N / 2, Pc, Pc, N / 2, N / 2, -S, S / 2, S / 2},
        {2.0 / 3.0, -ic, ic, B, -F, I, I, N / 2, -N / 2, -Pc, Pc, N / 2, -N / 2, S, S / 2, S / 2},
        {2.0 / 3.0, -ic, -ic, B, F, I, I, N / 2, N / 2, -Pc, -Pc, -N / 2, -N / 2, -S, S / 2, S / 2},
        {2.0 / 3.0, ic, -ic, B, -F, I, I, -N / 2, N / 2, Pc, -Pc, -N / 2, N / 2, S, S / 2, S / 2},
        {-0.5, 0, 0, D, 0, J, K, -N / 8, 0, Qc, 0, 0, R, 0, U, V},
        {-0.5, 0, 0, D, 0, K, J, 0, -N / 8, 0, Qc, R, 0, 0, V, U},
        {-0.5, 0, 0, D, 0, J, K, N / 8, 0, -Qc, 0, 0, -R, 0, U, V},
        {-0.5, 0, 0, D, 0, K, J, 0, N / 8, 0, -Qc, -R, 0, 0, V, U},
        {1.0 / 12, -jc, -jc, E, -F / 16, L, L, N / 16, N / 16, -Pc / 8, -Pc / 8, -R / 2, -R / 2, S / 4, S / 4, S / 4},
        {1.0 / 12, jc, -jc, E, F / 16, L, L, -N / 16, N / 16, Pc / 8, -Pc / 8, -R / 2, R / 2, -S / 4, S / 4, S / 4},
        {1.0 / 12, jc, jc, E, -F / 16, L, L, -N / 16, -N / 16, Pc / 8, Pc / 8, R / 2, R / 2, S / 4, S / 4, S / 4},
        {1.0 / 12, -jc, jc, E, F / 16, L, L, N / 16, -N / 16, -Pc / 8, Pc / 8, R / 2, -R / 2, -S / 4, S / 4, S / 4}};
    for (int a = 0; a < 16; ++a)
        for (int b = 0; b < 16; ++b) out[a][b] = m[a][b];
}

static void d2v16_eq_host(const Params &P, const double iM[16][16], double rho, double u, double v, double *eq) {
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
    for (int j = 0; j < 16; ++j) {
        double s = 0;
        for (int k = 0; k < 16; ++k) s += iM[j][k] * M[k];
        eq[j] = s;
    }
}

// Pseudopotential equilibrium at rest, eq(rho, 0, 0) (D2V16 through the
// inverse moment matrix, D2Q9PP w rho): the rest state of the FP32 storage.
void pp_rest_eq(const Params &P, const double iM[16][16], double rho, double *eq) {
    if (P.model == PP16) {
        d2v16_eq_host(P, iM, rho, 0.0, 0.0, eq);
    } else {
        for (int q = 0; q < 9; ++q) eq[q] = P.omega[q] * rho;
    }
}

// kind: 0 AC_Drop, 1 droplet heavy inside, 2 Rayleigh-Taylor, 3 SCMP_Drop, 4 density noise.
int host_init_state(const Params &P, const double iM[16][16], int kind, const double *params, int nparams,
                    uint64_t seed, std::vector<double> &f, std::vector<double> &h, std::vector<double> &aux) {
    const int nx = P.nx, ny = P.ny, Q = P.Q;
    const size_t n = (size_t)nx * ny;
    const bool ac = (P.model == AC || P.model == HCZ);
    if (ac && (kind < 0 || kind > 2)) return DUGKS_EINVAL;
    if (!ac && (kind < 3 || kind > 4)) return DUGKS_EINVAL;
    f.assign((size_t)Q * n, 0.0);
    h.clear();
    aux.assign((size_t)NFIELDS * n, 0.0);
    auto A = [&](int fld, int j, int i) -> double & { return aux[(size_t)fld * n + (size_t)j * nx + i]; };
    const double ChLength = (double)nx, Lx = (double)nx;
    // MacroQuantity init(Rho0,U0,V0,p0,T0,Lambda0,Mu0): everything else zero
    const double Rho0 = 1.0, U0 = 0.0, V0 = U0, p0 = 1, Mu0 = P.Tau0 * P.RT * Rho0;  // Mu0 = Nu0*Rho0
    (void)Mu0;
    if (ac) {
        h.assign((size_t)Q * n, 0.0);
        const double centerX = 0.5 * ChLength, centerY = 0.5 * ChLength;
        const double radius = (nparams >= 1 && params && params[0] >= 0) ? params[0] : 0.36 * ChLength;
        // Rayleigh-Taylor interface y = Lx (yc + amp cos(2 pi x / Lx)); optional params
        // {yc, amp, noise}: mean height and amplitude in units of Lx (default 2, 0.1), and
        // the amplitude of seeded uniform white noise added to phi (default 0)
        double rt_yc = 2.0, rt_amp = 0.1, rt_noise = 0.0;
        if (kind == 2 && params) {
            if (nparams >= 1) rt_yc = params[0];
            if (nparams >= 2) rt_amp = params[1];
            if (nparams >= 3) rt_noise = params[2];
        }
        uint64_t rng = seed;
        // Mu0 of the reference header, not Tau0*RT: the first step's tau is Mu0/(Rho*RT)
        const double mu0 = P.NuL * Rho0;  // NuL = Nu0 = Mu0/Rho0
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double x = i + 0.5, y = j + 0.5;
                double Phi;
                if (kind == 0) {  // AnalyticalPhiAC_Drop (Ark/Cpp/Preprocess.cpp:402-438)
                    Phi = 0.5 * (P.PhiL + P.PhiV) + 0.5 * (P.PhiL - P.PhiV) *
                          std::tanh((std::sqrt((x - centerX) * (x - centerX) + (y - centerY) * (y - centerY)) - radius) *
                                    2 / P.wI);
                } else if (kind == 1) {
                    const double r = std::sqrt((x - centerX) * (x - centerX) + (y - centerY) * (y - centerY));
                    Phi = 0.5 * (P.PhiL + P.PhiV) + 0.5 * (P.PhiL - P.PhiV) * std::tanh((radius - r) * 2 / P.wI);
                } else {
                    const double yi = Lx * (rt_yc + rt_amp * std::cos(2.0 * 3.141592653589793 * x / Lx));
                    Phi = 0.5 * (P.PhiL + P.PhiV) + 0.5 * (P.PhiL - P.PhiV) * std::tanh((y - yi) * 2 / P.wI);
                    if (rt_noise != 0.0) {
                        rng = rng * 6364136223846793005ULL + 1442695040888963407ULL;  // 64-bit LCG (Knuth MMIX)
                        const double u01 = (double)(rng >> 11) * (1.0 / 9007199254740992.0);
                        Phi += rt_noise * (2.0 * u01 - 1.0);
                    }
                }
                const double Rho = P.aPhi * (Phi) + P.bPhi;
                A(F_PHI, j, i) = Phi;
                A(F_RHO, j, i) = Rho;
                A(F_U, j, i) = U0;
                A(F_V, j, i) = V0;
                A(F_P, j, i) = p0;
                A(F_TAU, j, i) = mu0 / (Rho * P.RT);  // calcTau with Mu = Mu0
                // Update_phi_Eq at u = 0, zero forces; Tilde = Eq
                const double U = U0, V = V0, uu = U * U + V * V;
                for (int q = 0; q < Q; ++q) {
                    const double u1 = (P.xi_u[q] * U + P.xi_v[q] * V) / P.RT;
                    const double GAMMA = u1 + 0.5 * u1 * u1 - uu * P.Lambda0;
                    const size_t o = (size_t)q * n + (size_t)j * nx + i;
                    h[o] = P.omega[q] * (1.0 + u1) * (Phi);
                    if (P.model == AC)
                        f[o] = P.omega[q] * (p0 / P.RT + Rho * GAMMA) - (double)(!q) * p0 / P.RT;
                    else
                        f[o] = P.omega[q] * (p0 + Rho * GAMMA * P.RT);
                }
            }
        return DUGKS_OK;
    }
    // pseudopotential
    double rl = 2.4806E-1, rv = 4.5435E-2, prad = 0.25 * ChLength, rho0 = 0.2, amp = 0.01;
    if (kind == 3 && params) {
        if (nparams >= 1) rl = params[0];
        if (nparams >= 2) rv = params[1];
        if (nparams >= 3 && params[2] >= 0) prad = params[2];
    }
    if (kind == 4 && params) {
        if (nparams >= 1) rho0 = params[0];
        if (nparams >= 2) amp = params[1];
    }
    uint64_t st = seed;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const double x = i + 0.5, y = j + 0.5;
            double Rho;
            if (kind == 3) {
                Rho = 0.5 * (rl + rv) - 0.5 * (-rl + rv) *
                      std::tanh(2 * (std::sqrt((x - 0.5 * ChLength) * (x - 0.5 * ChLength) +
                                               (y - 0.5 * ChLength) * (y - 0.5 * ChLength)) - prad) / 5.0);
            } else {
                st = st * 6364136223846793005ULL + 1442695040888963407ULL;  // 64-bit LCG (Knuth MMIX)
                const double u01 = (double)(st >> 11) * (1.0 / 9007199254740992.0);
                Rho = rho0 * (1.0 + amp * (2.0 * u01 - 1.0));
            }
            A(F_RHO, j, i) = Rho;
            A(F_P, j, i) = Rho * P.RT;
            A(F_U, j, i) = U0;
            A(F_V, j, i) = V0;
            A(F_TAU, j, i) = P.Tau0;
            double eq[16];
            if (P.model == PP16) {
                d2v16_eq_host(P, iM, Rho, U0, V0, eq);
            } else {
                const double U = U0, V = V0, uu = U * U + V * V;
                for (int q = 0; q < Q; ++q) {
                    const double u1 = (P.xi_u[q] * U + P.xi_v[q] * V) / P.RT;
                    eq[q] = P.omega[q] * Rho * (1.0 + u1 + 0.5 * u1 * u1 - uu * P.Lambda0);
                }
            }
            for (int q = 0; q < Q; ++q) f[(size_t)q * n + (size_t)j * nx + i] = eq[q];
        }
    return DUGKS_OK;
}

}  // namespace dugks
