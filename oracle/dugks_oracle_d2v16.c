/* D2V16 equilibrium for the CPU restatement -- TEST INFRASTRUCTURE ONLY.
 *
 * The reference's D2V16 model (Ark/Lib/D2V16.cpp) does not compile against
 * its own headers, so there is no reference binary for it.  This file
 * restates its equilibrium: f_eq = M^-1 m(rho,u,v,T,p) with the 16x16
 * inverse moment matrix of Ark/Lib/D2V16.cpp:14-52 (built here from the same
 * closed-form coefficients A..V of c and e = (3+nK)c), the velocity set of
 * Ark/Lib/D2V16.cpp:53-66 and the moment vector Macro16 of
 * Ark/Lib/D2V16.cpp:125-145, evaluated at T = T0 and p = rho*R0*T0
 * (isothermal use with the pseudopotential force).  The table layout has to
 * match the reference; the code is this project's own.
 */
#include <math.h>
#include <string.h>

typedef struct orc_state orc_state;
/* accessors into the private state (defined in dugks_oracle.c via the same layout) */
#define MAXQ 16

struct orc_d2v16_view {
    double *xi_u, *xi_v, *omega, *xi2;
    double (*iM)[MAXQ];
    double R0, T0, MaSpan;
};

/* The state struct is private to dugks_oracle.c; it exposes the fields this
 * file needs through these two hooks. */
void orc_internal_view(orc_state *s, struct orc_d2v16_view *v);
void orc_internal_cview(const orc_state *s, struct orc_d2v16_view *v);

void orc_d2v16_setup(orc_state *s) {
    struct orc_d2v16_view vw;
    orc_internal_view(s, &vw);
    const double nK = 0;
    const double c = vw.MaSpan, e = (3.0 + nK) * vw.MaSpan;
    const double c2 = c * c, e2 = e * e, c2e2 = c2 * e2;
    const double A = 1.0 / (4.0 * e2), B = (-21.0 * c2 - e2) / (48.0 * c2e2),
                 D = (7.0 * c2 + e2) / (32.0 * c2e2), E = (-3.0 * c2 - e2) / (96.0 * c2e2),
                 F = 1.0 / (3.0 * c2), G = (3.0 * c2 - 5.0 * e2) / (4.0 * e2 * (e2 - 3.0 * c2)),
                 H = 3.0 * (c2 + e2) / (4.0 * e2 * (e2 - 3.0 * c2)),
                 I = (21.0 * c2 - 11.0 * e2) / (48.0 * c2e2),
                 J = (21.0 * c2 * c2 - 32.0 * c2e2 + 11.0 * e2 * e2) / (32.0 * c2e2 * (e2 - 3.0 * c2)),
                 K = (21.0 * c2 * c2 - 36.0 * c2e2 + 7.0 * e2 * e2) / (32.0 * c2e2 * (e2 - 3.0 * c2)),
                 L = (3.0 * c2 - 5.0 * e2) / (96.0 * c2e2), N = 1.0 / (2.0 * c * e2),
                 P = (3.0 * c2 - e2) / (12.0 * c2e2 * c), Qc = (c2 + e2) / (16.0 * c2e2 * c),
                 R = (c2 - e2) / (16.0 * c2e2 * c), S = 1.0 / (24.0 * c2 * c2),
                 T = 1.0 / (4.0 * c2 * (e2 - 3.0 * c2)),
                 U = (c2 - e2) / (32.0 * c2 * c2 * (e2 - 3.0 * c2)),
                 V = (5.0 * c2 - e2) / (32.0 * c2 * c2 * (e2 - 3.0 * c2));
    const double m[16][16] = {
        {0, 0, 0, A, 0, G, H, N, 0, -N, 0, 0, -N, 0, T, -T},
        {0, 0, 0, A, 0, H, G, 0, N, 0, -N, -N, 0, 0, -T, T},
        {0, 0, 0, A, 0, G, H, -N, 0, N, 0, 0, N, 0, T, -T},
        {0, 0, 0, A, 0, H, G, 0, -N, 0, N, N, 0, 0, -T, T},
        {2.0 / 3.0, 1.0 / (3.0 * c), 1.0 / (3.0 * c), B, F, I, I, -N / 2, -N / 2, P, P, N / 2, N / 2, -S, S / 2, S / 2},
        {2.0 / 3.0, -1.0 / (3.0 * c), 1.0 / (3.0 * c), B, -F, I, I, N / 2, -N / 2, -P, P, N / 2, -N / 2, S, S / 2, S / 2},
        {2.0 / 3.0, -1.0 / (3.0 * c), -1.0 / (3.0 * c), B, F, I, I, N / 2, N / 2, -P, -P, -N / 2, -N / 2, -S, S / 2, S / 2},
        {2.0 / 3.0, 1.0 / (3.0 * c), -1.0 / (3.0 * c), B, -F, I, I, -N / 2, N / 2, P, -P, -N / 2, N / 2, S, S / 2, S / 2},
        {-0.5, 0, 0, D, 0, J, K, -N / 8, 0, Qc, 0, 0, R, 0, U, V},
        {-0.5, 0, 0, D, 0, K, J, 0, -N / 8, 0, Qc, R, 0, 0, V, U},
        {-0.5, 0, 0, D, 0, J, K, N / 8, 0, -Qc, 0, 0, -R, 0, U, V},
        {-0.5, 0, 0, D, 0, K, J, 0, N / 8, 0, -Qc, -R, 0, 0, V, U},
        {1.0 / 12, -1.0 / (24 * c), -1.0 / (24 * c), E, -F / 16, L, L, N / 16, N / 16, -P / 8, -P / 8, -R / 2, -R / 2, S / 4, S / 4, S / 4},
        {1.0 / 12, 1.0 / (24 * c), -1.0 / (24 * c), E, F / 16, L, L, -N / 16, N / 16, P / 8, -P / 8, -R / 2, R / 2, -S / 4, S / 4, S / 4},
        {1.0 / 12, 1.0 / (24 * c), 1.0 / (24 * c), E, -F / 16, L, L, -N / 16, -N / 16, P / 8, P / 8, R / 2, R / 2, S / 4, S / 4, S / 4},
        {1.0 / 12, -1.0 / (24 * c), 1.0 / (24 * c), E, F / 16, L, L, N / 16, -N / 16, -P / 8, P / 8, R / 2, -R / 2, -S / 4, S / 4, S / 4}};
    memcpy(vw.iM, m, sizeof m);
    const double su[16] = {1, 0, -1, 0, 1, -1, -1, 1, 2, 0, -2, 0, 2, -2, -2, 2};
    const double sv[16] = {0, 1, 0, -1, 1, 1, -1, -1, 0, 2, 0, -2, 2, 2, -2, -2};
    const double r2[16] = {0, 0, 0, 0, 2, 2, 2, 2, 4, 4, 4, 4, 8, 8, 8, 8};
    for (int q = 0; q < 16; ++q) {
        vw.xi_u[q] = su[q] * c;   /* {c,0,-c,0,...,2c,...}: su*c is exact for su in {0,±1,±2} */
        vw.xi_v[q] = sv[q] * c;
        vw.xi2[q] = q < 4 ? c2 + e2 : r2[q] * c2;
        vw.omega[q] = 0.0;
    }
}

/* Macro16 (Ark/Lib/D2V16.cpp:125-145) with degrees = 3+nK = 3, then M^-1. */
void orc_d2v16_eq(const orc_state *s, double rho, double u, double v, double *eq) {
    struct orc_d2v16_view vw;
    orc_internal_cview(s, &vw);
    const double degrees = 3.0, degPlus2 = degrees + 2.0;
    const double T = vw.T0;
    const double p = rho * vw.R0 * T;
    double M[16];
    const double u2 = u * u, v2 = v * v, RT = vw.R0 * T;
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
        double sum = 0;
        for (int k = 0; k < 16; ++k) sum += vw.iM[j][k] * M[k];
        eq[j] = sum;
    }
}
