/* CPU restatement of the reference DUGKS step -- TEST INFRASTRUCTURE ONLY.
 * See dugks_oracle.h.  Build with -O2 -ffp-contract=off (no FMA contraction:
 * the reference is compiled the same way for the bit-exact pin).
 *
 * Grid: nx*ny unit cells, periodic in x; in y periodic or bounce-back walls
 * with one ghost row on each side (Ark/Cpp/Boundary.cpp:38-139).  Fields
 * that a stencil reads across the y boundary live in "extended" arrays of
 * ny+2 rows (row 0 and row ny+1 are the ghost/wrap rows).
 *
 * Faces: xf(i,j) is the west face of cell (i,j) (owner (i-1,j), neighbour
 * (i,j), normal +x); yf(i,j) the south face of cell (i,j) (owner (i,j-1),
 * neighbour (i,j), normal +y), j = 0..ny (rows 0 and ny are walls when
 * y_walls).  The reference computes each periodic boundary face twice, once
 * from each side (Ark/Cpp/DUGKS2DSolver.cpp:224-229); on this mesh the two
 * copies are bitwise equal (exact geometry, orientation-independent
 * formulas), so each face is computed once.
 */
#include "dugks_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXQ 16

struct orc_state {
    orc_inputs in;
    int nx, ny, Q, has_h;
    /* derived constants */
    double R0, T0, RT, Lambda0, Rho0, U0, V0, p0, Mu0, Nu0, Tau0, CFL, MinL, ChLength;
    double MaxU, MaSpan, dt, hDt, Lx, Ly, DeltaX, DeltaY, _2dx, _2dy;
    double M_Phi, Cn, wI, Sigma, Beta, Kappa, PhiL, PhiV, RhoL, RhoV, aPhi, bPhi;
    double MuL, MuV, NuL, NuV, TauMass, Gx, Gy, centerX, centerY, radius, Kp;
    double aTP, bTP;
    double h_aBP, h_bBP, h_cBP, h_ah, h_bh, h_ch; /* constant phase-field factors */
    double T_r, T_CS, aCS, Kpp;                   /* pseudopotential EOS */
    double xi_u[MAXQ], xi_v[MAXQ], omega[MAXQ], xi2[MAXQ];
    int bb[MAXQ];
    /* D2V16 inverse moment matrix */
    double iM[MAXQ][MAXQ];
    /* state */
    double *f, *h;                    /* tilde [Q][ny][nx] */
    double *rho, *u, *v, *p, *tauf;   /* [ny][nx] */
    double *prevphiu, *prevphiv, *scg;
    double *phi, *phix, *phiy, *rhox, *rhoy, *fx, *fy, *psi; /* extended [ny+2][nx] */
    /* scratch */
    double *bf, *bh;                  /* BarP, extended [Q][ny+2][nx] */
    double *Fxf, *Fxh;                /* x-face flux [Q][ny][nx] */
    double *Fyf, *Fyh;                /* y-face flux [Q][ny+1][nx] */
    /* pseudopotential face state (D2Q9PP/D2V16): previous face force, face psi */
    double *xfFx, *xfFy, *yfFx, *yfFy; /* x: [ny][nx]; y: [ny+1][nx] */
    double *xpsi, *ypsi, *xscg, *yscg, *xrho, *yrho, *xu, *yu, *xv, *yv; /* pass-1 results */
    /* UW: cell gradients of BarP, extended [Q][ny+2][nx]; fluxes of the periodic
     * boundary faces computed from the low side (owner in column 0 / row 0) */
    double *gfx, *gfy, *ghx, *ghy;
    double *Fxlo_f, *Fxlo_h;          /* [Q][ny] */
    double *Fylo_f, *Fylo_h;          /* [Q][nx] */
    /* NEE walls: the cell equilibria and sources of the wall rows (bottom, top) [2][Q][nx] */
    double *wEqf, *wSof, *wEqh, *wSoh;
    long step;
};

/* ------------------------------------------------------------------ */
static inline int wrapx(const orc_state *s, int i) { return (i + s->nx) % s->nx; }
#define C(s, j, i) ((size_t)(j) * (s)->nx + (i))                 /* cell [ny][nx] */
#define E(s, j, i) ((size_t)((j) + 1) * (s)->nx + (i))           /* extended row j in -1..ny */
#define DQ(s, arr, q, j, i) (arr)[(size_t)(q) * (s)->ny * (s)->nx + C(s, j, i)]
#define BQ(s, arr, q, j, i) (arr)[(size_t)(q) * ((s)->ny + 2) * (s)->nx + E(s, j, i)]
#define XQ(s, arr, q, j, i) (arr)[(size_t)(q) * (s)->ny * (s)->nx + C(s, j, i)]
#define YQ(s, arr, q, j, i) (arr)[(size_t)(q) * ((s)->ny + 1) * (s)->nx + C(s, j, i)]

static inline void SetZero(double *d) { if (*d < 1.0E-14 && *d > -1.0E-14) *d = 0.0; }

/* Carnahan-Starling with b = 4 (Ark/Lib/nonidealEoS.h:114-118) */
static inline double CarnahanStarling(const orc_state *s, double rho) {
    return rho * s->R0 * s->T_CS * (1.0 + rho + rho * rho - rho * rho * rho) /
               ((1.0 - rho) * (1.0 - rho) * (1.0 - rho)) -
           s->aCS * rho * rho;
}

/* Ark/Header/Macroscopic.h:64-68 */
static inline void calcPsi(const orc_state *s, double rho, double p, double *scg, double *psi) {
    double G = (double)((p > rho * s->RT) - (p < rho * s->RT));
    *scg = G;
    *psi = sqrt(2 * (p - rho * s->RT) / G);
}

/* ------------------------------------------------------------------ */
static void derive(orc_state *s) {
    const orc_inputs *in = &s->in;
    int D2V16 = in->model == ORC_PP16;
    /* Ark/Constant/ZeroReference.h */
    s->ChLength = (double)in->nx;
    s->MinL = s->ChLength / in->nx;
    s->Lx = (double)in->nx - 0.0;
    s->Ly = (double)in->ny - 0.0;
    s->DeltaX = s->Lx / in->nx;
    s->DeltaY = s->Ly / in->ny;
    s->T0 = 1.0 / 3;
    s->R0 = 1.0;
    s->RT = s->R0 * s->T0;
    s->Lambda0 = 1 / (2.0 * s->R0 * s->T0);
    s->Rho0 = 1.0;
    s->U0 = 0.0;
    s->V0 = s->U0;
    s->p0 = 1;
    s->Mu0 = in->Mu0;
    s->Nu0 = s->Mu0 / s->Rho0;
    s->Tau0 = s->Nu0 / s->RT;
    /* Ark/Lib/D2Q9.h, Ark/Lib/D2V16.h */
    if (D2V16) {
        s->MaSpan = in->d2v16_c;
        s->MaxU = 2 * s->MaSpan * sqrt(2.0);
    } else {
        s->MaxU = sqrt(3.0 * s->RT);
        s->MaSpan = sqrt(3.0 * s->RT);
    }
    /* Ark/Constant/ZeroNamespace.h */
    s->CFL = 0.5;
    s->dt = s->CFL > 0.0 ? s->CFL * s->MinL / s->MaxU : 1.0E-4;
    s->hDt = 0.5 * s->dt;
    s->M_Phi = in->M_Phi;
    s->Cn = in->W / s->ChLength;
    s->wI = s->ChLength * s->Cn;
    s->Sigma = in->Sigma;
    s->Beta = 12.0 * s->Sigma / s->wI;
    s->Kappa = 3.0 * s->Sigma * s->wI / 2;
    s->PhiL = 1.0;
    s->PhiV = 0.0;
    s->RhoL = in->RhoL;
    s->RhoV = in->RhoV;
    s->MuL = s->Nu0 * s->RhoL;
    s->MuV = s->Nu0 * s->RhoV;
    s->NuL = s->Nu0;
    s->NuV = s->Nu0;
    s->aPhi = (s->RhoL - s->RhoV) / (s->PhiL - s->PhiV);
    s->bPhi = s->RhoV - s->aPhi * s->PhiV;
    s->Gx = 0.0;
    s->Gy = in->gravity ? in->Gy : 0.0;
    s->TauMass = s->M_Phi / s->RT;
    s->centerX = 0.5 * s->ChLength;
    s->centerY = 0.5 * s->ChLength;
    s->radius = in->radius < 0 ? 0.36 * s->ChLength : in->radius;
    s->Kp = s->RT * 9 / 5.0;                       /* Ark/Lib/D2Q9AC.cpp:32 */
    s->_2dx = 2.0 * s->DeltaX;                     /* Ark/Lib/GradSchemeBasic.h:7-11 */
    s->_2dy = 2.0 * s->DeltaY;
    s->aTP = 4.0 / 3.0;                            /* Ark/Cpp/DUGKS2DSolver.cpp:12 */
    s->bTP = 1.0 / 3.0;
    /* constant phase-field relaxation (Cell_2D.cpp:120-125, Face_2D.cpp:306-311) */
    {
        double tau = s->TauMass;
        s->h_aBP = (2.0 * tau - s->hDt) / (2.0 * tau + s->dt);
        s->h_bBP = 1.0 - s->h_aBP;
        s->h_cBP = tau * s->h_bBP;
        s->h_ah = 2.0 * tau / (2.0 * tau + s->hDt);
        s->h_bh = 1.0 - s->h_ah;
        s->h_ch = tau * s->h_bh;
    }
    /* Ark/Lib/nonidealEoS.h */
    s->T_r = in->Tr;
    s->aCS = in->aCS;
    s->T_CS = s->T_r * in->Tc_CS;
    /* velocity sets */
    if (!D2V16) {
        static const double xu[9] = {0, 1, 1, 0, -1, -1, -1, 0, 1};
        static const double xv[9] = {0, 0, 1, 1, 1, 0, -1, -1, -1};
        static const int bb[9] = {0, 5, 6, 7, 8, 1, 2, 3, 4};
        double w[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 36.0, 1.0 / 9.0, 1.0 / 36.0,
                       1.0 / 9.0, 1.0 / 36.0, 1.0 / 9.0, 1.0 / 36.0};
        s->Q = 9;
        for (int q = 0; q < 9; ++q) {
            s->xi_u[q] = s->MaSpan * xu[q];
            s->xi_v[q] = s->MaSpan * xv[q];
            s->omega[q] = w[q];
            s->bb[q] = bb[q];
        }
    }
}

/* ---------------------------- D2V16 ------------------------------- */
/* Equilibrium through the 16x16 inverse moment matrix of Ark/Lib/D2V16.cpp:11-74
 * (c = MaSpan, e = (3+nK)c, nK = 0) and Macro16 (Ark/Lib/D2V16.cpp:125-145)
 * with T = T0 (isothermal pseudopotential use).  Implemented in
 * dugks_oracle_d2v16.c. */
void orc_d2v16_setup(orc_state *s);
void orc_d2v16_eq(const orc_state *s, double rho, double u, double v, double *eq);

struct orc_d2v16_view {
    double *xi_u, *xi_v, *omega, *xi2;
    double (*iM)[MAXQ];
    double R0, T0, MaSpan;
};
void orc_internal_view(orc_state *s, struct orc_d2v16_view *v) {
    v->xi_u = s->xi_u; v->xi_v = s->xi_v; v->omega = s->omega; v->xi2 = s->xi2;
    v->iM = s->iM; v->R0 = s->R0; v->T0 = s->T0; v->MaSpan = s->MaSpan;
}
void orc_internal_cview(const orc_state *s, struct orc_d2v16_view *v) {
    orc_internal_view((orc_state *)s, v);
}

/* ------------------------------------------------------------------ */
static void *xalloc(size_t n) {
    void *p = calloc(n ? n : 1, sizeof(double));
    return p;
}

orc_state *orc_create(const orc_inputs *in) {
    if (in->nx < 3 || in->ny < 3) return NULL;
    orc_state *s = (orc_state *)calloc(1, sizeof(orc_state));
    s->in = *in;
    s->nx = in->nx;
    s->ny = in->ny;
    derive(s);
    if (in->model == ORC_PP16) {
        s->Q = 16;
        orc_d2v16_setup(s);
    }
    s->has_h = (in->model == ORC_AC || in->model == ORC_HCZ);
    size_t nc = (size_t)s->nx * s->ny, ne = (size_t)s->nx * (s->ny + 2), ny1 = (size_t)s->nx * (s->ny + 1);
    int Q = s->Q;
    s->f = xalloc(Q * nc);
    s->h = xalloc(Q * nc);
    s->rho = xalloc(nc); s->u = xalloc(nc); s->v = xalloc(nc); s->p = xalloc(nc); s->tauf = xalloc(nc);
    s->prevphiu = xalloc(nc); s->prevphiv = xalloc(nc); s->scg = xalloc(nc);
    s->phi = xalloc(ne); s->phix = xalloc(ne); s->phiy = xalloc(ne); s->rhox = xalloc(ne);
    s->rhoy = xalloc(ne); s->fx = xalloc(ne); s->fy = xalloc(ne); s->psi = xalloc(ne);
    s->bf = xalloc(Q * ne); s->bh = xalloc(Q * ne);
    s->Fxf = xalloc(Q * nc); s->Fxh = xalloc(Q * nc);
    s->Fyf = xalloc(Q * ny1); s->Fyh = xalloc(Q * ny1);
    s->xfFx = xalloc(nc); s->xfFy = xalloc(nc); s->yfFx = xalloc(ny1); s->yfFy = xalloc(ny1);
    s->xpsi = xalloc(nc); s->ypsi = xalloc(ny1); s->xscg = xalloc(nc); s->yscg = xalloc(ny1);
    s->xrho = xalloc(nc); s->yrho = xalloc(ny1); s->xu = xalloc(nc); s->yu = xalloc(ny1);
    s->xv = xalloc(nc); s->yv = xalloc(ny1);
    if (in->nee) {
        if (!s->has_h || !in->y_walls) {
            orc_destroy(s);
            return NULL;
        }
        s->wEqf = xalloc((size_t)2 * Q * s->nx); s->wSof = xalloc((size_t)2 * Q * s->nx);
        s->wEqh = xalloc((size_t)2 * Q * s->nx); s->wSoh = xalloc((size_t)2 * Q * s->nx);
    }
    if (in->uw) {
        if (!s->has_h || in->y_walls) {  /* the reference's UW with walls reads unwritten shadow-cell gradients */
            orc_destroy(s);
            return NULL;
        }
        s->gfx = xalloc(Q * ne); s->gfy = xalloc(Q * ne); s->ghx = xalloc(Q * ne); s->ghy = xalloc(Q * ne);
        s->Fxlo_f = xalloc((size_t)Q * s->ny); s->Fxlo_h = xalloc((size_t)Q * s->ny);
        s->Fylo_f = xalloc((size_t)Q * s->nx); s->Fylo_h = xalloc((size_t)Q * s->nx);
    }

    const int nx = s->nx, ny = s->ny;
    if (s->has_h) {
        /* AC_Drop-style init (Ark/Cpp/Preprocess.cpp:705-760, AC_RisingBubble 761-823):
         * MsQ = (Rho0,U0,V0,p0,T0,Lambda0,Mu0), phase-field profile, tau from Mu0. */
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double x = i + 0.5, y = j + 0.5, Phi;
                if (in->init == ORC_INIT_AC_DROP) {
                    Phi = 0.5 * (s->PhiL + s->PhiV) + 0.5 * (s->PhiL - s->PhiV) *
                          tanh((sqrt((x - s->centerX) * (x - s->centerX) + (y - s->centerY) * (y - s->centerY)) - s->radius) * 2 / s->wI);
                } else if (in->init == ORC_INIT_AC_DROP_INSIDE) {
                    double r = sqrt((x - s->centerX) * (x - s->centerX) + (y - s->centerY) * (y - s->centerY));
                    Phi = 0.5 * (s->PhiL + s->PhiV) + 0.5 * (s->PhiL - s->PhiV) * tanh((s->radius - r) * 2 / s->wI);
                } else {
                    double yi = s->Lx * (2.0 + 0.1 * cos(2.0 * 3.141592653589793 * x / s->Lx));
                    Phi = 0.5 * (s->PhiL + s->PhiV) + 0.5 * (s->PhiL - s->PhiV) * tanh((y - yi) * 2 / s->wI);
                }
                double Rho = s->aPhi * (Phi) + s->bPhi;
                size_t c = C(s, j, i), e = E(s, j, i);
                s->phi[e] = Phi;
                s->rho[c] = Rho;
                s->u[c] = s->U0;
                s->v[c] = s->V0;
                s->p[c] = s->p0;
                s->tauf[c] = s->Mu0 / (Rho * s->RT);    /* calcTau with Mu = Mu0 */
            }
        /* Update_phi_Eq with all forces zero; Tilde = Eq */
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t c = C(s, j, i), e = E(s, j, i);
                double U = s->u[c], V = s->v[c], uu = U * U + V * V;
                for (int q = 0; q < Q; ++q) {
                    double u1 = (s->xi_u[q] * U + s->xi_v[q] * V) / s->RT;
                    double GAMMA = u1 + 0.5 * u1 * u1 - uu * s->Lambda0;
                    DQ(s, s->h, q, j, i) = s->omega[q] * (1.0 + u1) * (s->phi[e]);
                    if (in->model == ORC_AC)
                        DQ(s, s->f, q, j, i) = s->omega[q] * (s->p[c] / s->RT + s->rho[c] * GAMMA) -
                                               (double)(!q) * s->p[c] / s->RT;
                    else
                        DQ(s, s->f, q, j, i) = s->omega[q] * (s->p[c] + s->rho[c] * GAMMA * s->RT);
                }
            }
    } else {
        /* pseudopotential: SCMP_Drop (Ark/Cpp/Preprocess.cpp:337-401) or seeded noise */
        uint64_t st = in->seed;
        double PRhoL = in->PP_RhoL, PRhoV = in->PP_RhoV;
        double prad = in->PP_radius < 0 ? 0.25 * s->ChLength : in->PP_radius;
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double x = i + 0.5, y = j + 0.5, Rho;
                if (in->init == ORC_INIT_SCMP_DROP) {
                    Rho = 0.5 * (PRhoL + PRhoV) - 0.5 * (-PRhoL + PRhoV) *
                          tanh(2 * (sqrt((x - 0.5 * s->ChLength) * (x - 0.5 * s->ChLength) +
                                         (y - 0.5 * s->ChLength) * (y - 0.5 * s->ChLength)) - prad) / 5.0);
                } else {
                    st = st * 6364136223846793005ULL + 1442695040888963407ULL;
                    double uu01 = (double)(st >> 11) * (1.0 / 9007199254740992.0);
                    Rho = in->noise_rho0 * (1.0 + in->noise_amp * (2.0 * uu01 - 1.0));
                }
                size_t c = C(s, j, i);
                s->rho[c] = Rho;
                s->p[c] = Rho * s->RT;
                s->u[c] = s->U0;
                s->v[c] = s->V0;
                s->tauf[c] = s->Tau0;
            }
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t c = C(s, j, i);
                double eq[MAXQ];
                if (in->model == ORC_PP16) {
                    orc_d2v16_eq(s, s->rho[c], s->u[c], s->v[c], eq);
                } else {
                    double U = s->u[c], V = s->v[c], uu = U * U + V * V;
                    for (int q = 0; q < Q; ++q) {
                        double u1 = (s->xi_u[q] * U + s->xi_v[q] * V) / s->RT;
                        eq[q] = s->omega[q] * s->rho[c] * (1.0 + u1 + 0.5 * u1 * u1 - uu * s->Lambda0);
                    }
                }
                for (int q = 0; q < Q; ++q) DQ(s, s->f, q, j, i) = eq[q];
            }
    }
    s->step = 0;
    return s;
}

void orc_destroy(orc_state *s) {
    if (!s) return;
    double **all[] = {&s->f, &s->h, &s->rho, &s->u, &s->v, &s->p, &s->tauf, &s->prevphiu, &s->prevphiv,
                      &s->scg, &s->phi, &s->phix, &s->phiy, &s->rhox, &s->rhoy, &s->fx, &s->fy, &s->psi,
                      &s->bf, &s->bh, &s->Fxf, &s->Fxh, &s->Fyf, &s->Fyh, &s->xfFx, &s->xfFy, &s->yfFx,
                      &s->yfFy, &s->xpsi, &s->ypsi, &s->xscg, &s->yscg, &s->xrho, &s->yrho, &s->xu,
                      &s->yu, &s->xv, &s->yv, &s->gfx, &s->gfy, &s->ghx, &s->ghy, &s->Fxlo_f, &s->Fxlo_h,
                      &s->Fylo_f, &s->Fylo_h, &s->wEqf, &s->wSof, &s->wEqh, &s->wSoh};
    for (size_t k = 0; k < sizeof all / sizeof all[0]; ++k) free(*all[k]);
    free(s);
}

int orc_nq(const orc_state *s) { return s->Q; }
long orc_steps_done(const orc_state *s) { return s->step; }

/* ------------------------- ghost / wrap rows ----------------------- */
static void wrap_rows(orc_state *s, double *ext) {
    int nx = s->nx, ny = s->ny;
    memcpy(ext + E(s, -1, 0), ext + E(s, ny - 1, 0), sizeof(double) * nx);
    memcpy(ext + E(s, ny, 0), ext + E(s, 0, 0), sizeof(double) * nx);
}
/* ghost = 2*first - second (Ark/Cpp/Boundary.cpp:38-63, int 2 and 2.0 alike) */
static void extrap_rows(orc_state *s, double *ext) {
    int nx = s->nx, ny = s->ny;
    for (int i = 0; i < nx; ++i) {
        ext[E(s, -1, i)] = 2.0 * ext[E(s, 0, i)] - ext[E(s, 1, i)];
        ext[E(s, ny, i)] = 2.0 * ext[E(s, ny - 1, i)] - ext[E(s, ny - 2, i)];
    }
}
static void fill_rows(orc_state *s, double *ext) {
    if (s->in.y_walls) extrap_rows(s, ext); else wrap_rows(s, ext);
}

/* ------------------------------ P1 -------------------------------- */
/* Update_phi_Eq + Update_DVDF_Source + Update_phi_BP for one cell
 * (Ark/Lib/D2Q9AC.cpp:69-105,331-344; Ark/Lib/D2Q9HCZ.cpp:54-92,244-257;
 *  Ark/Lib/D2Q9PP.cpp:51-62,137-145; Ark/Cpp/DUGKS2DSolver.cpp:379-401) */
static void cell_barp(orc_state *s, int i, int j) {
    size_t c = C(s, j, i), e = E(s, j, i);
    const int model = s->in.model, Q = s->Q;
    double U = s->u[c], V = s->v[c], Rho = s->rho[c], p = s->p[c];
    double Fx = s->fx[e], Fy = s->fy[e];
    double tau = s->tauf[c];
    double aBP = (2.0 * tau - s->hDt) / (2.0 * tau + s->dt), bBP = 1.0 - aBP, cBP = tau * bBP;
    if (model == ORC_AC || model == ORC_HCZ) {
        double Phi = s->phi[e], Rho_x = s->rhox[e], Rho_y = s->rhoy[e];
        double Phi_x = s->phix[e], Phi_y = s->phiy[e];
        double uu = U * U + V * V;
        for (int q = 0; q < Q; ++q) {
            double xu = s->xi_u[q], xv = s->xi_v[q], w = s->omega[q];
            double u1 = (xu * U + xv * V) / s->RT;
            double GAMMA = u1 + 0.5 * u1 * u1 - uu * s->Lambda0;
            double hEq = w * (1.0 + u1) * (Phi);
            double fEq, fSo;
            if (model == ORC_AC) {
                fEq = w * (p / s->RT + Rho * GAMMA) - (double)(!q) * p / s->RT;
                fSo = w * ((1 + GAMMA) * ((xu - U) * (Fx) + (xv - V) * (Fy)) / s->RT +
                           GAMMA * ((xu - U) * (Rho_x) + (xv - V) * (Rho_y)));
            } else {
                fEq = w * (p + Rho * GAMMA * s->RT);
                fSo = w * ((1 + GAMMA) * ((xu - U) * (Fx) + (xv - V) * (Fy)) +
                           GAMMA * s->RT * ((xu - U) * (Rho_x) + (xv - V) * (Rho_y)));
            }
            double hSo = ((Phi_x) * (xu) + (Phi_y) * xv) * w;
            if (s->in.nee && (j == 0 || j == s->ny - 1)) { /* kept for Wall_3_NEE */
                size_t o = ((size_t)(j == 0 ? 0 : 1) * Q + q) * s->nx + i;
                s->wEqf[o] = fEq;
                s->wSof[o] = fSo;
                s->wEqh[o] = hEq;
                s->wSoh[o] = hSo;
            }
            BQ(s, s->bh, q, j, i) = s->h_aBP * DQ(s, s->h, q, j, i) + s->h_bBP * hEq + s->h_cBP * hSo;
            double b = aBP * DQ(s, s->f, q, j, i) + bBP * fEq;
            b += cBP * fSo;
            BQ(s, s->bf, q, j, i) = b;
        }
    } else {
        double eq[MAXQ];
        if (model == ORC_PP16) {
            orc_d2v16_eq(s, Rho, U, V, eq);
        } else {
            double uu = U * U + V * V;
            for (int q = 0; q < Q; ++q) {
                double u1 = (s->xi_u[q] * U + s->xi_v[q] * V) / s->RT;
                eq[q] = s->omega[q] * Rho * (1.0 + u1 + 0.5 * u1 * u1 - uu * s->Lambda0);
            }
        }
        for (int q = 0; q < Q; ++q) {
            double So = (Fx * (s->xi_u[q] - U) + Fy * (s->xi_v[q] - V)) * eq[q] / (Rho * s->RT);
            double b = aBP * DQ(s, s->f, q, j, i) + bBP * eq[q];
            b += cBP * So;
            BQ(s, s->bf, q, j, i) = b;
        }
    }
}

/* --------------------------- face pass ---------------------------- */
/* CD_Interior_phi_Bh (Ark/Cpp/DUGKS2DSolver.cpp:604-687) in the canonical
 * orientation: x-face owner L = (i-1,j), neighbour R = (i,j); y-face owner
 * B = (i,j-1), neighbour T = (i,j).  Writes the face distribution BhDt. */
static void face_bh(const orc_state *s, const double *B, int xface, int i, int j, double *out) {
    const int Q = s->Q;
    int im = wrapx(s, i - 1), ip = wrapx(s, i + 1);
    for (int q = 0; q < Q; ++q) {
        double gx, gy, o, n;
        if (xface) {
            o = BQ(s, B, q, j, im);
            n = BQ(s, B, q, j, i);
            double SL = BQ(s, B, q, j - 1, im), SR = BQ(s, B, q, j - 1, i);
            double NL = BQ(s, B, q, j + 1, im), NR = BQ(s, B, q, j + 1, i);
            gy = (0.5 * (NR - SR) + 0.5 * (NL - SL)) / (2 * s->DeltaY);
            gx = (o - n) / (-s->DeltaX);
        } else {
            o = BQ(s, B, q, j - 1, i);
            n = BQ(s, B, q, j, i);
            double WB = BQ(s, B, q, j - 1, im), EB = BQ(s, B, q, j - 1, ip);
            double WT = BQ(s, B, q, j, im), ET = BQ(s, B, q, j, ip);
            gx = (0.5 * (WT - ET) + 0.5 * (WB - EB)) / (2 * (-s->DeltaX));
            gy = (o - n) / (-s->DeltaY);
        }
        out[q] = 0.5 * (o + n) - s->hDt * (gx * (s->xi_u[q]) + gy * s->xi_v[q]);
    }
}

/* UW flux scheme (_FLUX_SCHEME_UW_ARK), periodic grids.  Cell gradients of
 * BarP, Grad_VS_6points (Ark/Cpp/GradScheme.cpp:205-218,
 * Ark/Lib/GradSchemeBasic.h:95-126): apsi = 4, bpsi = 1, C0..C3 = E,N,W,S,
 * D0..D3 = NE,NW,SW,SE. */
static void cell_grad6(orc_state *s, const double *B, double *GX, double *GY, int i, int j) {
    int im = wrapx(s, i - 1), ip = wrapx(s, i + 1);
    for (int q = 0; q < s->Q; ++q) {
        double E_ = BQ(s, B, q, j, ip), W_ = BQ(s, B, q, j, im);
        double N_ = BQ(s, B, q, j + 1, i), S_ = BQ(s, B, q, j - 1, i);
        double D0 = BQ(s, B, q, j + 1, ip), D1 = BQ(s, B, q, j + 1, im);
        double D2 = BQ(s, B, q, j - 1, im), D3 = BQ(s, B, q, j - 1, ip);
        BQ(s, GX, q, j, i) = (4.0 * (E_ - W_) + 1.0 * (D0 - D1 + D3 - D2)) / (s->_2dx * 6);
        BQ(s, GY, q, j, i) = (4.0 * (N_ - S_) + 1.0 * (D0 - D3 + D1 - D2)) / (s->_2dy * 6);
    }
}

/* Grad_VS_LS (Ark/Cpp/GradScheme.cpp:219-231 -> Ark/Lib/GradSchemeBasic.h:127-152): the
 * least-squares gradient, sum over C0..C3 = E,N,W,S of w_k (B_k - B_c), then the inverse
 * 2x2 matrix of Grad_LSMatrix (:13-75).  On unit cells the cell centres are exact
 * (i + 1/2, j + 1/2; periodic shadows offset by exactly Lx, Ly), so wdx = {1,0,-1,0},
 * wdy = {0,1,0,-1} and the inverse is {{0.5,-0},{-0,0.5}}; the reference's products and
 * sums are all kept, zero terms included. */
static void cell_grad_ls(orc_state *s, const double *B, double *GX, double *GY, int i, int j) {
    int im = wrapx(s, i - 1), ip = wrapx(s, i + 1);
    static const double wdx[4] = {1.0, 0.0, -1.0, 0.0}, wdy[4] = {0.0, 1.0, 0.0, -1.0};
    for (int q = 0; q < s->Q; ++q) {
        double c = BQ(s, B, q, j, i);
        double nb[4] = {BQ(s, B, q, j, ip), BQ(s, B, q, j + 1, i), BQ(s, B, q, j, im), BQ(s, B, q, j - 1, i)};
        double sx = 0.0, sy = 0.0;
        for (int k = 0; k < 4; ++k) {
            sx += wdx[k] * (nb[k] - c);
            sy += wdy[k] * (nb[k] - c);
        }
        BQ(s, GX, q, j, i) = 0.5 * sx + -0.0 * sy;
        BQ(s, GY, q, j, i) = -0.0 * sx + 0.5 * sy;
    }
}

/* Grad_VS_4points (Ark/Cpp/GradScheme.cpp:191-204 -> Ark/Lib/GradSchemeBasic.h:76-94):
 * (C0 - C2) / _2dx and (C1 - C3) / _2dy */
static void cell_grad4(orc_state *s, const double *B, double *GX, double *GY, int i, int j) {
    int im = wrapx(s, i - 1), ip = wrapx(s, i + 1);
    for (int q = 0; q < s->Q; ++q) {
        BQ(s, GX, q, j, i) = (BQ(s, B, q, j, ip) - BQ(s, B, q, j, im)) / s->_2dx;
        BQ(s, GY, q, j, i) = (BQ(s, B, q, j + 1, i) - BQ(s, B, q, j - 1, i)) / s->_2dy;
    }
}

/* the cell gradient of the UW scheme: in->uw 1 6-point, 2 least squares, 3 4-point */
static void cell_grad(orc_state *s, const double *B, double *GX, double *GY, int i, int j) {
    if (s->in.uw == 2) cell_grad_ls(s, B, GX, GY, i, j);
    else if (s->in.uw == 3) cell_grad4(s, B, GX, GY, i, j);
    else cell_grad6(s, B, GX, GY, i, j);
}

/* UW_Interior_phi_Bh (Ark/Cpp/DUGKS2DSolver.cpp:558-603), chosen by the sign of
 * xi.n dS (:689-706): the upwind cell's BarP + (dx BarP_x + dy BarP_y) with
 * (dx, dy) = x_f - hDt xi - x_c, the two cells averaged (owner first) along the
 * face.  Canonical orientation as face_bh: o = (i-1,j) or (i,j-1), n = (i,j),
 * normal +x / +y; cell centres relative to the face at -1/2 and +1/2 along the
 * normal (exact, as the reference's coordinates on the unit grid).  lo: the
 * periodic boundary face as the reference computes it from the low side
 * (owner n inside the domain, normal -x / -y). */
static void face_uw(const orc_state *s, const double *B, const double *GX, const double *GY, int xface, int i,
                    int j, int lo, double *out) {
    int io = xface ? wrapx(s, i - 1) : i, jo = xface ? j : j - 1;
    double xo = xface ? -0.5 : 0.0, yo = xface ? 0.0 : -0.5;
    double xn = xface ? 0.5 : 0.0, yn = xface ? 0.0 : 0.5;
    for (int q = 0; q < s->Q; ++q) {
        double xsh = 0.0 - s->hDt * s->xi_u[q], ysh = 0.0 - s->hDt * s->xi_v[q];
        double Bo = BQ(s, B, q, jo, io), Bn = BQ(s, B, q, j, i);
        double Xo = (xsh - xo) * BQ(s, GX, q, jo, io) + (ysh - yo) * BQ(s, GY, q, jo, io);
        double Xn = (xsh - xn) * BQ(s, GX, q, j, i) + (ysh - yn) * BQ(s, GY, q, j, i);
        double xin = xface ? s->xi_u[q] : s->xi_v[q];
        double sgn = lo ? -xin : xin;
        double ow = lo ? Bn : Bo, owX = lo ? Xn : Xo, ne = lo ? Bo : Bn, neX = lo ? Xo : Xn;
        if (sgn > 0) out[q] = ow + owX;
        else if (sgn < 0) out[q] = ne + neX;
        else out[q] = (ow + owX + ne + neX) / 2;
    }
}

/* Face moments, equilibrium, source and flux for the Allen-Cahn models
 * (Ark/Lib/D2Q9AC.cpp:106-144,232-329,345-358; Ark/Lib/D2Q9HCZ.cpp:93-131,
 *  183-242,258-271; Ark/Cpp/DUGKS2DSolver.cpp:402-441; Ark/Cpp/Boundary.cpp:118-139).
 * avg[6] = owner/neighbour averages of Phi_x', Phi_y', Rho_x, Rho_y, Fx, Fy.
 * wall: 0 none, -1 bottom wall (owner above), +1 top wall (owner below).
 * Output: fluxes already multiplied by xi.n dS for the +x / +y normal. */
static void face_flux_ac(const orc_state *s, const double *bhf, const double *bhh, const double *avg,
                         int xface, int wall, double *outf, double *outh) {
    const int Q = s->Q, model = s->in.model;
    double Phi_x = avg[0], Phi_y = avg[1], Rho_x = avg[2], Rho_y = avg[3], Fx = avg[4], Fy = avg[5];
    double Phi = 0, sumf = 0;
    for (int q = 0; q < Q; ++q) Phi += bhh[q];
    for (int q = 0; q < Q; ++q) sumf += bhf[q];
    double Rho = s->aPhi * Phi + s->bPhi;
    double U, V, p, Mu;
    if (model == ORC_AC) {
        U = 0.0;
        V = 0.0;
        p = sumf - bhf[0];
        p += (0.5 * s->hDt * (Rho_x * U + Rho_y * V) - s->omega[0] * Rho * (U * U + V * V) * s->Lambda0);
        p *= s->Kp;
        Mu = Rho * s->RT * s->Tau0;
    } else {
        double su = 0, sv = 0;
        for (int q = 0; q < Q; ++q) su += bhf[q] * s->xi_u[q];
        for (int q = 0; q < Q; ++q) sv += bhf[q] * s->xi_v[q];
        U = su / (Rho * s->RT);
        V = sv / (Rho * s->RT);
        U += 0.5 * s->hDt * Fx / (Rho * s->RT);
        V += 0.5 * s->hDt * Fy / (Rho * s->RT);
        p = sumf + 0.5 * s->hDt * s->RT * (Rho_x * U + Rho_y * V);
        Mu = s->NuV + (Phi - s->PhiV) * (s->NuL - s->NuV);
        Mu *= Rho;
    }
    double tauh = Mu / (Rho * s->RT);
    double ah = 2.0 * tauh / (2.0 * tauh + s->hDt), bh = 1.0 - ah, ch = tauh * bh;
    double uu = U * U + V * V;
    double hf[MAXQ], hh[MAXQ];
    for (int q = 0; q < Q; ++q) {
        double xu = s->xi_u[q], xv = s->xi_v[q], w = s->omega[q];
        double u1 = (xu * U + xv * V) / s->RT;
        double GAMMA = u1 + 0.5 * u1 * u1 - uu * s->Lambda0;
        double hEq = w * Phi * (1.0 + u1);
        double fEq, fSo;
        if (model == ORC_AC) {
            fEq = w * (p / s->RT + Rho * GAMMA) - (double)(!q) * p / s->RT;
            fSo = w * ((1 + GAMMA) * ((xu - U) * Fx + (xv - V) * (Fy)) / s->RT +
                       GAMMA * ((xu - U) * Rho_x + (xv - V) * (Rho_y)));
        } else {
            fEq = w * (p + Rho * s->RT * GAMMA);
            fSo = w * ((1 + GAMMA) * ((xu - U) * Fx + (xv - V) * (Fy)) +
                       GAMMA * s->RT * ((xu - U) * Rho_x + (xv - V) * (Rho_y)));
        }
        double hSo = (Phi_x * xu + Phi_y * xv) * w;
        hh[q] = s->h_ah * bhh[q] + s->h_bh * hEq + s->h_ch * hSo;
        double t = ah * bhf[q] + bh * fEq;
        t += ch * fSo;
        hf[q] = t;
    }
    if (wall) {
        /* bounce-back on directions entering the domain (xi.n_out < 0) */
        for (int q = 0; q < Q; ++q) {
            double xn = wall < 0 ? -s->xi_v[q] : s->xi_v[q];
            if (xn < 0) {
                hh[q] = hh[s->bb[q]];
                hf[q] = hf[s->bb[q]];
            }
        }
    }
    for (int q = 0; q < Q; ++q) {
        double xn = xface ? s->xi_u[q] : s->xi_v[q];
        outf[q] = hf[q] * xn;
        outh[q] = hh[q] * xn;
    }
}

/* Wall_3_NEE (Ark/Cpp/Boundary.cpp:140-184) on the wall face of column i; side 0 the
 * bottom wall (owner (i,0), the face 0.5 below its centre), 1 the top wall (owner
 * (i,ny-1)).  The face's U, V keep the initial value 0 of its MsQh (the routine never
 * sets them); phi and rho are the owner's extrapolated with its Phi_x/Phi_y (the
 * phase-field source vector after MacroSource) and Rho_x/Rho_y; p is the owner's;
 * Update_phi_Eqh at those moments, the owner's non-equilibrium part
 * (Tilde - Eq + hDt So) scaled by 2 tau / (2 tau + dt), then bounce-back. */
static void face_nee(const orc_state *s, int i, int side, double *outf, double *outh) {
    const int Q = s->Q, model = s->in.model, jc = side ? s->ny - 1 : 0;
    size_t c = C(s, jc, i), e = E(s, jc, i);
    double dxw = 0.0, dyw = side ? 0.5 : -0.5; /* face centre - cell centre */
    double Phi = s->phi[e] + s->phix[e] * dxw + s->phiy[e] * dyw;
    double Rho = s->rho[c] + s->rhox[e] * dxw + s->rhoy[e] * dyw;
    double p = s->p[c], U = 0.0, V = 0.0;
    double uu = U * U + V * V;
    double hNEq = 2.0 * s->TauMass / (2.0 * s->TauMass + s->dt);
    double fNEq = 2.0 * s->tauf[c] / (2.0 * s->tauf[c] + s->dt);
    double hf[MAXQ], hh[MAXQ];
    for (int q = 0; q < Q; ++q) {
        double xu = s->xi_u[q], xv = s->xi_v[q], w = s->omega[q];
        double u1 = (xu * U + xv * V) / s->RT;
        double GAMMA = u1 + 0.5 * u1 * u1 - uu * s->Lambda0;
        double hEq = w * Phi * (1.0 + u1);
        double fEq = model == ORC_AC ? w * (p / s->RT + Rho * GAMMA) - (double)(!q) * p / s->RT
                                     : w * (p + Rho * s->RT * GAMMA);
        size_t o = ((size_t)side * Q + q) * s->nx + i;
        hh[q] = hEq + hNEq * (DQ(s, s->h, q, jc, i) - s->wEqh[o] + s->hDt * s->wSoh[o]);
        hf[q] = fEq + fNEq * (DQ(s, s->f, q, jc, i) - s->wEqf[o] + s->hDt * s->wSof[o]);
    }
    for (int q = 0; q < Q; ++q) { /* Wall_3_BB */
        double xn = side ? s->xi_v[q] : -s->xi_v[q];
        if (xn < 0) {
            hh[q] = hh[s->bb[q]];
            hf[q] = hf[s->bb[q]];
        }
    }
    for (int q = 0; q < Q; ++q) {
        outf[q] = hf[q] * s->xi_v[q];
        outh[q] = hh[q] * s->xi_v[q];
    }
}

/* ----------------------- pseudopotential faces -------------------- */
static void face_pp_pass1(orc_state *s, const double *bhf, double prevFx, double prevFy,
                          double *rho, double *u, double *v, double *scg, double *psi) {
    const int Q = s->Q;
    double R = 0, su = 0, sv = 0;
    for (int q = 0; q < Q; ++q) R += bhf[q];
    for (int q = 0; q < Q; ++q) su += bhf[q] * s->xi_u[q];
    for (int q = 0; q < Q; ++q) sv += bhf[q] * s->xi_v[q];
    double U = su / R, V = sv / R;
    U += 0.5 * s->hDt * prevFx / R;          /* Ark/Lib/D2Q9PP.cpp:110-136 */
    V += 0.5 * s->hDt * prevFy / R;
    double p = 1.0 * CarnahanStarling(s, R); /* Ark/Cpp/PseudoP.cpp:23-30 */
    *rho = R;
    *u = U;
    *v = V;
    calcPsi(s, R, p, scg, psi);
}

static void face_pp_flux(const orc_state *s, const double *bhf, double R, double U, double V,
                         double Fx, double Fy, int xface, double *outf) {
    const int Q = s->Q;
    double eq[MAXQ];
    if (s->in.model == ORC_PP16) {
        orc_d2v16_eq(s, R, U, V, eq);
    } else {
        double uu = U * U + V * V;
        for (int q = 0; q < Q; ++q) {
            double u1 = (s->xi_u[q] * U + s->xi_v[q] * V) / s->RT;
            eq[q] = s->omega[q] * R * (1.0 + u1 + 0.5 * u1 * u1 - uu * s->Lambda0);
        }
    }
    double tauh = s->Tau0;
    double ah = 2.0 * tauh / (2.0 * tauh + s->hDt), bh = 1.0 - ah, ch = tauh * bh;
    for (int q = 0; q < Q; ++q) {
        double So = (Fx * (s->xi_u[q] - U) + Fy * (s->xi_v[q] - V)) * eq[q] / (R * s->RT);
        double t = ah * bhf[q] + bh * eq[q];
        t += ch * So;
        outf[q] = t * (xface ? s->xi_u[q] : s->xi_v[q]);
    }
}

/* 8-neighbour isotropic gradient (Ark/Lib/GradSchemeBasic.h:153-208) on a
 * periodic nx*rows lattice given by a row accessor. */
static inline double iso_gx(double E_, double W_, double NE, double NW, double SE, double SW, double d2) {
    return (4 * ((E_) - (W_)) + 1 * ((NE) - (NW) + (SE) - (SW))) / (d2 * 6);
}
static inline double iso_gy(double N_, double S_, double NE, double NW, double SE, double SW, double d2) {
    return (4 * ((N_) - (S_)) + 1 * ((NE) - (SE) + (NW) - (SW))) / (d2 * 6);
}

/* ------------------------------ step ------------------------------ */
static void one_step(orc_state *s) {
    const int nx = s->nx, ny = s->ny, Q = s->Q, model = s->in.model;
    const int walls = s->in.y_walls;
    const int AC = (model == ORC_AC || model == ORC_HCZ);
    /* P1: collision pre-step */
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) cell_barp(s, i, j);
    /* P2: ghost / wrap rows of BarP and of the macro fields read by faces */
    for (int q = 0; q < Q; ++q) {
        fill_rows(s, s->bf + (size_t)q * (ny + 2) * nx);
        if (AC) fill_rows(s, s->bh + (size_t)q * (ny + 2) * nx);
    }
    if (AC) {
        double *mf[] = {s->phi, s->phix, s->phiy, s->rhox, s->rhoy, s->fx, s->fy};
        for (int k = 0; k < 7; ++k) fill_rows(s, mf[k]);
    }
    const int uw = s->in.uw;
    if (uw) { /* UW: cell gradients of BarP (Ark/Cpp/DUGKS2DSolver.cpp:196-205) */
#pragma omp parallel for schedule(static)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                cell_grad(s, s->bf, s->gfx, s->gfy, i, j);
                cell_grad(s, s->bh, s->ghx, s->ghy, i, j);
            }
        for (int q = 0; q < Q; ++q) {
            double *g[] = {s->gfx, s->gfy, s->ghx, s->ghy};
            for (int k = 0; k < 4; ++k) fill_rows(s, g[k] + (size_t)q * (ny + 2) * nx);
        }
    }
    /* P4 + P6: faces */
    if (AC) {
#pragma omp parallel for schedule(static)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double bf[MAXQ], bh[MAXQ], of[MAXQ], oh[MAXQ], avg[6];
                int im = wrapx(s, i - 1);
                size_t a = E(s, j, im), b = E(s, j, i);
                avg[0] = 0.5 * ((s->phix[a]) + (s->phix[b]));
                avg[1] = 0.5 * ((s->phiy[a]) + (s->phiy[b]));
                avg[2] = 0.5 * ((s->rhox[a]) + (s->rhox[b]));
                avg[3] = 0.5 * ((s->rhoy[a]) + (s->rhoy[b]));
                avg[4] = 0.5 * ((s->fx[a]) + (s->fx[b]));
                avg[5] = 0.5 * ((s->fy[a]) + (s->fy[b]));
                if (uw) {
                    face_uw(s, s->bf, s->gfx, s->gfy, 1, i, j, 0, bf);
                    face_uw(s, s->bh, s->ghx, s->ghy, 1, i, j, 0, bh);
                } else {
                    face_bh(s, s->bf, 1, i, j, bf);
                    face_bh(s, s->bh, 1, i, j, bh);
                }
                face_flux_ac(s, bf, bh, avg, 1, 0, of, oh);
                for (int q = 0; q < Q; ++q) {
                    XQ(s, s->Fxf, q, j, i) = of[q];
                    XQ(s, s->Fxh, q, j, i) = oh[q];
                }
                if (uw && i == 0) { /* the left boundary face of the reference (owner (0,j)) */
                    face_uw(s, s->bf, s->gfx, s->gfy, 1, i, j, 1, bf);
                    face_uw(s, s->bh, s->ghx, s->ghy, 1, i, j, 1, bh);
                    face_flux_ac(s, bf, bh, avg, 1, 0, of, oh);
                    for (int q = 0; q < Q; ++q) {
                        s->Fxlo_f[(size_t)q * ny + j] = of[q];
                        s->Fxlo_h[(size_t)q * ny + j] = oh[q];
                    }
                }
            }
        int jy1 = walls ? ny + 1 : ny;
#pragma omp parallel for schedule(static)
        for (int j = 0; j < jy1; ++j)
            for (int i = 0; i < nx; ++i) {
                double bf[MAXQ], bh[MAXQ], of[MAXQ], oh[MAXQ], avg[6];
                size_t a = E(s, j - 1, i), b = E(s, j, i);
                avg[0] = 0.5 * ((s->phix[a]) + (s->phix[b]));
                avg[1] = 0.5 * ((s->phiy[a]) + (s->phiy[b]));
                avg[2] = 0.5 * ((s->rhox[a]) + (s->rhox[b]));
                avg[3] = 0.5 * ((s->rhoy[a]) + (s->rhoy[b]));
                avg[4] = 0.5 * ((s->fx[a]) + (s->fx[b]));
                avg[5] = 0.5 * ((s->fy[a]) + (s->fy[b]));
                if (uw) {
                    face_uw(s, s->bf, s->gfx, s->gfy, 0, i, j, 0, bf);
                    face_uw(s, s->bh, s->ghx, s->ghy, 0, i, j, 0, bh);
                } else {
                    face_bh(s, s->bf, 0, i, j, bf);
                    face_bh(s, s->bh, 0, i, j, bh);
                }
                int wall = walls ? (j == 0 ? -1 : (j == ny ? 1 : 0)) : 0;
                if (wall && s->in.nee) face_nee(s, i, wall > 0, of, oh);
                else face_flux_ac(s, bf, bh, avg, 0, wall, of, oh);
                for (int q = 0; q < Q; ++q) {
                    YQ(s, s->Fyf, q, j, i) = of[q];
                    YQ(s, s->Fyh, q, j, i) = oh[q];
                }
                if (uw && j == 0) { /* the bottom boundary face of the reference (owner (i,0)) */
                    face_uw(s, s->bf, s->gfx, s->gfy, 0, i, j, 1, bf);
                    face_uw(s, s->bh, s->ghx, s->ghy, 0, i, j, 1, bh);
                    face_flux_ac(s, bf, bh, avg, 0, 0, of, oh);
                    for (int q = 0; q < Q; ++q) {
                        s->Fylo_f[(size_t)q * nx + i] = of[q];
                        s->Fylo_h[(size_t)q * nx + i] = oh[q];
                    }
                }
            }
        if (!walls) {
            for (int q = 0; q < Q; ++q)
                for (int i = 0; i < nx; ++i) {
                    YQ(s, s->Fyf, q, ny, i) = YQ(s, s->Fyf, q, 0, i);
                    YQ(s, s->Fyh, q, ny, i) = YQ(s, s->Fyh, q, 0, i);
                }
        }
    } else {
        /* pseudopotential: pass 1 over all faces, then face force and flux */
#pragma omp parallel for schedule(static)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double bf[MAXQ];
                size_t c = C(s, j, i);
                face_bh(s, s->bf, 1, i, j, bf);
                face_pp_pass1(s, bf, s->xfFx[c], s->xfFy[c], &s->xrho[c], &s->xu[c], &s->xv[c],
                              &s->xscg[c], &s->xpsi[c]);
                face_bh(s, s->bf, 0, i, j, bf);
                face_pp_pass1(s, bf, s->yfFx[c], s->yfFy[c], &s->yrho[c], &s->yu[c], &s->yv[c],
                              &s->yscg[c], &s->ypsi[c]);
            }
#pragma omp parallel for schedule(static)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double bf[MAXQ], of[MAXQ];
                size_t c = C(s, j, i);
                int im = wrapx(s, i - 1), ip = wrapx(s, i + 1);
                int jm = (j - 1 + ny) % ny, jp = (j + 1) % ny;
                const double *X = s->xpsi, *Y = s->ypsi;
#define P_(A, jj, ii) (A)[C(s, jj, ii)]
                double gx = iso_gx(P_(X, j, ip), P_(X, j, im), P_(X, jp, ip), P_(X, jp, im), P_(X, jm, ip), P_(X, jm, im), s->_2dx);
                double gy = iso_gy(P_(X, jp, i), P_(X, jm, i), P_(X, jp, ip), P_(X, jp, im), P_(X, jm, ip), P_(X, jm, im), s->_2dy);
                double k = -s->xscg[c] * s->xpsi[c];
                s->xfFx[c] = gx * k;
                s->xfFy[c] = gy * k;
                face_bh(s, s->bf, 1, i, j, bf);
                face_pp_flux(s, bf, s->xrho[c], s->xu[c], s->xv[c], s->xfFx[c], s->xfFy[c], 1, of);
                for (int q = 0; q < Q; ++q) XQ(s, s->Fxf, q, j, i) = of[q];
                gx = iso_gx(P_(Y, j, ip), P_(Y, j, im), P_(Y, jp, ip), P_(Y, jp, im), P_(Y, jm, ip), P_(Y, jm, im), s->_2dx);
                gy = iso_gy(P_(Y, jp, i), P_(Y, jm, i), P_(Y, jp, ip), P_(Y, jp, im), P_(Y, jm, ip), P_(Y, jm, im), s->_2dy);
                k = -s->yscg[c] * s->ypsi[c];
                s->yfFx[c] = gx * k;
                s->yfFy[c] = gy * k;
                face_bh(s, s->bf, 0, i, j, bf);
                face_pp_flux(s, bf, s->yrho[c], s->yu[c], s->yv[c], s->yfFx[c], s->yfFy[c], 0, of);
                for (int q = 0; q < Q; ++q) YQ(s, s->Fyf, q, j, i) = of[q];
#undef P_
            }
        for (int q = 0; q < Q; ++q)
            for (int i = 0; i < nx; ++i) YQ(s, s->Fyf, q, ny, i) = YQ(s, s->Fyf, q, 0, i);
    }
    /* P8: finite-volume update (Ark/Cpp/DUGKS2DSolver.cpp:748-792), faces E,N,W,S */
    const double dtV = s->dt / (s->DeltaX * s->DeltaY);
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            int ip = wrapx(s, i + 1);
            /* UW: the west face of column 0 / south face of row 0 are the low-side boundary faces */
            int xlo = uw && i == 0, ylo = uw && j == 0;
            for (int q = 0; q < Q; ++q) {
                double S = 0.0;
                S += -1 * XQ(s, s->Fxf, q, j, ip);
                S += -1 * YQ(s, s->Fyf, q, j + 1, i);
                S += 1 * (xlo ? s->Fxlo_f[(size_t)q * ny + j] : XQ(s, s->Fxf, q, j, i));
                S += 1 * (ylo ? s->Fylo_f[(size_t)q * nx + i] : YQ(s, s->Fyf, q, j, i));
                DQ(s, s->f, q, j, i) = s->aTP * BQ(s, s->bf, q, j, i) - s->bTP * DQ(s, s->f, q, j, i) + dtV * S;
                if (AC) {
                    double H = 0.0;
                    H += -1 * XQ(s, s->Fxh, q, j, ip);
                    H += -1 * YQ(s, s->Fyh, q, j + 1, i);
                    H += 1 * (xlo ? s->Fxlo_h[(size_t)q * ny + j] : XQ(s, s->Fxh, q, j, i));
                    H += 1 * (ylo ? s->Fylo_h[(size_t)q * nx + i] : YQ(s, s->Fyh, q, j, i));
                    DQ(s, s->h, q, j, i) = s->aTP * BQ(s, s->bh, q, j, i) - s->bTP * DQ(s, s->h, q, j, i) + dtV * H;
                }
            }
        }
    /* P9: cell macros */
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            size_t c = C(s, j, i), e = E(s, j, i);
            double sumf = 0;
            for (int q = 0; q < Q; ++q) sumf += DQ(s, s->f, q, j, i);
            if (AC) {
                double Phi = 0;
                for (int q = 0; q < Q; ++q) Phi += DQ(s, s->h, q, j, i);
                double Rho = s->aPhi * Phi + s->bPhi, U, V, p, Mu;
                s->phi[e] = Phi;
                if (model == ORC_AC) {
                    U = 0.0;
                    V = 0.0;
                    p = sumf - DQ(s, s->f, 0, j, i);
                    p += (s->hDt * (s->rhox[e] * U + s->rhoy[e] * V) - Rho * s->omega[0] * (U * U + V * V) * s->Lambda0);
                    p *= s->Kp;
                    Mu = Rho * s->RT * s->Tau0;
                } else {
                    double su = 0, sv = 0;
                    for (int q = 0; q < Q; ++q) su += DQ(s, s->f, q, j, i) * s->xi_u[q];
                    for (int q = 0; q < Q; ++q) sv += DQ(s, s->f, q, j, i) * s->xi_v[q];
                    U = (su) / (Rho * s->RT);
                    V = (sv) / (Rho * s->RT);
                    U += s->hDt * (s->fx[e]) / (Rho * s->RT);
                    V += s->hDt * (s->fy[e]) / (Rho * s->RT);
                    p = sumf + s->hDt * (s->rhox[e] * U + s->rhoy[e] * V) * s->RT;
                    Mu = s->NuV + (Phi - s->PhiV) * (s->NuL - s->NuV);
                    Mu *= Rho;
                }
                s->rho[c] = Rho;
                s->u[c] = U;
                s->v[c] = V;
                s->p[c] = p;
                s->tauf[c] = Mu / (Rho * s->RT);
            } else {
                double su = 0, sv = 0;
                for (int q = 0; q < Q; ++q) su += DQ(s, s->f, q, j, i) * s->xi_u[q];
                for (int q = 0; q < Q; ++q) sv += DQ(s, s->f, q, j, i) * s->xi_v[q];
                double Rho = sumf;
                double U = (su) / Rho, V = (sv) / Rho;
                U += s->hDt * s->fx[e] / Rho;
                V += s->hDt * s->fy[e] / Rho;
                double p = 1.0 * CarnahanStarling(s, Rho);
                s->rho[c] = Rho;
                s->u[c] = U;
                s->v[c] = V;
                s->p[c] = p;
                calcPsi(s, Rho, p, &s->scg[c], &s->psi[e]);
            }
        }
    /* P10 / P11: Allen-Cahn sources (Ark/Cpp/SourceM.cpp:15-62, Ark/Cpp/GradScheme.cpp:347-376)
     * or pseudopotential cell force (Ark/Cpp/PseudoP.cpp:31-38). */
    if (AC) {
        if (!walls) wrap_rows(s, s->phi); /* walls keep the P2 ghost phi (previous step) */
#pragma omp parallel for schedule(static)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t c = C(s, j, i), e = E(s, j, i);
                int im = wrapx(s, i - 1), ip = wrapx(s, i + 1);
                const double *P = s->phi;
                double Ec = P[E(s, j, ip)], Wc = P[E(s, j, im)], Nc = P[E(s, j + 1, i)], Sc = P[E(s, j - 1, i)];
                double NE = P[E(s, j + 1, ip)], NW = P[E(s, j + 1, im)], SW = P[E(s, j - 1, im)], SE = P[E(s, j - 1, ip)];
                double Phi = P[e];
                double Phi_x = iso_gx(Ec, Wc, NE, NW, SE, SW, s->_2dx);
                double Phi_y = iso_gy(Nc, Sc, NE, NW, SE, SW, s->_2dy);
                double lap = (4 * ((Ec) + (Nc) + (Wc) + (Sc)) + (NE + NW + SW + SE) - 20 * (Phi)) /
                             (6 * s->MinL * s->MinL);
                SetZero(&Phi_x);
                SetZero(&Phi_y);
                double F = 2 * s->Beta * (Phi - s->PhiL) * (Phi - s->PhiV) * (2 * Phi - s->PhiL - s->PhiV) -
                           s->Kappa * lap;
                double Rho = s->rho[c], U = s->u[c], V = s->v[c];
                double Rho_x = s->aPhi * Phi_x, Rho_y = s->aPhi * Phi_y;
                double Fx = F * Phi_x, Fy = F * Phi_y;
                if (s->in.gravity) Fy -= s->Gy * (Rho - s->RhoL);
                double L = sqrt(Phi_x * Phi_x + Phi_y * Phi_y);
                double dU = Phi * U - s->prevphiu[c], dV = Phi * V - s->prevphiv[c];
                double sx, sy;
                if (L != 0) {
                    double tmp = -4 * (Phi - s->PhiL) * (Phi - s->PhiV) / (s->wI * (s->PhiL - s->PhiV));
                    sx = (Phi_x) * tmp / L + dU / (s->RT * s->dt);
                    sy = (Phi_y) * tmp / L + dV / (s->RT * s->dt);
                } else {
                    sx = dU / (s->RT * s->dt);
                    sy = dV / (s->RT * s->dt);
                }
                /* results go to scratch first: neighbours still read phi only */
                s->Fxf[c] = sx;
                s->Fxh[c] = sy;
                s->rhox[e] = Rho_x;
                s->rhoy[e] = Rho_y;
                s->fx[e] = Fx;
                s->fy[e] = Fy;
                s->prevphiu[c] = (Phi) * (U);
                s->prevphiv[c] = (Phi) * (V);
            }
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                s->phix[E(s, j, i)] = s->Fxf[C(s, j, i)];
                s->phiy[E(s, j, i)] = s->Fxh[C(s, j, i)];
            }
    } else {
        wrap_rows(s, s->psi);
#pragma omp parallel for schedule(static)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t c = C(s, j, i), e = E(s, j, i);
                int im = wrapx(s, i - 1), ip = wrapx(s, i + 1);
                const double *P = s->psi;
                double gx = iso_gx(P[E(s, j, ip)], P[E(s, j, im)], P[E(s, j + 1, ip)], P[E(s, j + 1, im)],
                                   P[E(s, j - 1, ip)], P[E(s, j - 1, im)], s->_2dx);
                double gy = iso_gy(P[E(s, j + 1, i)], P[E(s, j - 1, i)], P[E(s, j + 1, ip)], P[E(s, j + 1, im)],
                                   P[E(s, j - 1, ip)], P[E(s, j - 1, im)], s->_2dy);
                double k = -s->scg[c] * P[e];
                s->fx[e] = gx * k;
                s->fy[e] = gy * k;
            }
    }
    s->step++;
}

void orc_step(orc_state *s, int nsteps, int nthreads) {
#ifdef _OPENMP
    int old = omp_get_max_threads();
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    for (int k = 0; k < nsteps; ++k) one_step(s);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(old);
#endif
    (void)nthreads;
}

/* ------------------------------ access ---------------------------- */
static int field_ptr(const orc_state *s, const char *name, double **base, int *ext, int *q) {
    *ext = 0;
    *q = -1;
    struct { const char *n; double *p; int e; } tab[] = {
        {"rho", s->rho, 0}, {"u", s->u, 0}, {"v", s->v, 0}, {"p", s->p, 0}, {"tauf", s->tauf, 0},
        {"prevphiu", s->prevphiu, 0}, {"prevphiv", s->prevphiv, 0}, {"scg", s->scg, 0},
        {"phi", s->phi, 1}, {"phix", s->phix, 1}, {"phiy", s->phiy, 1}, {"rhox", s->rhox, 1},
        {"rhoy", s->rhoy, 1}, {"fx", s->fx, 1}, {"fy", s->fy, 1}, {"psi", s->psi, 1}};
    for (size_t k = 0; k < sizeof tab / sizeof tab[0]; ++k)
        if (!strcmp(tab[k].n, name)) {
            *base = tab[k].p;
            *ext = tab[k].e;
            return 0;
        }
    if ((name[0] == 'f' || name[0] == 'h') && name[1] >= '0' && name[1] <= '9') {
        int qq = atoi(name + 1);
        if (qq < 0 || qq >= s->Q) return -1;
        if (name[0] == 'h' && !s->has_h) return -1;
        *base = name[0] == 'f' ? s->f : s->h;
        *q = qq;
        return 0;
    }
    return -1;
}

int orc_get(const orc_state *s, const char *name, double *out) {
    double *b;
    int ext, q;
    if (field_ptr(s, name, &b, &ext, &q)) return -1;
    for (int j = 0; j < s->ny; ++j)
        for (int i = 0; i < s->nx; ++i)
            out[C(s, j, i)] = q >= 0 ? b[(size_t)q * s->ny * s->nx + C(s, j, i)] : (ext ? b[E(s, j, i)] : b[C(s, j, i)]);
    return 0;
}

int orc_set(orc_state *s, const char *name, const double *in) {
    double *b;
    int ext, q;
    if (field_ptr(s, name, &b, &ext, &q)) return -1;
    for (int j = 0; j < s->ny; ++j)
        for (int i = 0; i < s->nx; ++i) {
            double v = in[C(s, j, i)];
            if (q >= 0) b[(size_t)q * s->ny * s->nx + C(s, j, i)] = v;
            else if (ext) b[E(s, j, i)] = v;
            else b[C(s, j, i)] = v;
        }
    return 0;
}

double orc_const(const orc_state *s, const char *name) {
    struct { const char *n; double v; } tab[] = {
        {"dt", s->dt}, {"hDt", s->hDt}, {"RT", s->RT}, {"Lambda0", s->Lambda0}, {"Tau0", s->Tau0},
        {"Kp", s->Kp}, {"aPhi", s->aPhi}, {"bPhi", s->bPhi}, {"Beta", s->Beta}, {"Kappa", s->Kappa},
        {"wI", s->wI}, {"TauMass", s->TauMass}, {"NuL", s->NuL}, {"NuV", s->NuV}, {"Gy", s->Gy},
        {"MaSpan", s->MaSpan}, {"T_CS", s->T_CS}, {"radius", s->radius}};
    for (size_t k = 0; k < sizeof tab / sizeof tab[0]; ++k)
        if (!strcmp(tab[k].n, name)) return tab[k].v;
    return NAN;
}

int orc_velocities(const orc_state *s, double *xi_u, double *xi_v, double *xi2) {
    for (int q = 0; q < s->Q; ++q) {
        xi_u[q] = s->xi_u[q];
        xi_v[q] = s->xi_v[q];
        xi2[q] = s->xi2[q];
    }
    return s->Q;
}

int orc_d2v16_equilibrium(const orc_state *s, double rho, double u, double v, double *eq) {
    if (s->in.model != ORC_PP16) return -1;
    orc_d2v16_eq(s, rho, u, v, eq);
    return 0;
}

void orc_sums(const orc_state *s, double *sum_rho, double *sum_phi) {
    double a = 0, b = 0;
    for (int j = 0; j < s->ny; ++j)
        for (int i = 0; i < s->nx; ++i) {
            a += s->rho[C(s, j, i)];
            if (s->has_h) b += s->phi[E(s, j, i)];
        }
    *sum_rho = a;
    *sum_phi = b;
}
