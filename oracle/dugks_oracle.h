/* CPU restatement of the reference DUGKS step -- TEST INFRASTRUCTURE ONLY.
 *
 * This is the oracle the GPU path is checked against.  It restates, on a
 * structured SoA grid, the per-cell and per-face functions of the reference
 * solver in the reference's own arithmetic order (compile with
 * -ffp-contract=off), so that on the same inputs it reproduces the reference
 * bit for bit; tests/test_oracle_vs_reference.py pins that against dumps of
 * the unmodified reference built by oracle/ref/build_ref.py and against the
 * committed fixtures in tests/golden/.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this library.  The product path never links or calls it.
 */
#ifndef DUGKS_ORACLE_H
#define DUGKS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_AC = 0, ORC_HCZ = 1, ORC_PP9 = 2, ORC_PP16 = 3 };
enum { ORC_INIT_AC_DROP = 0, ORC_INIT_AC_DROP_INSIDE = 1, ORC_INIT_AC_RT = 2,
       ORC_INIT_SCMP_DROP = 3, ORC_INIT_PP_NOISE = 4 };

/* Primary inputs; every derived constant is computed from these with the
 * expressions of Ark/Constant/ZeroReference.h and Ark/Constant/ZeroNamespace.h. */
typedef struct orc_inputs {
    int model, nx, ny, y_walls, gravity, init;
    double Mu0, M_Phi, W, Sigma, RhoL, RhoV, Gy, radius;   /* radius < 0: 0.36*ChLength */
    double Tr, aCS, Tc_CS, PP_RhoL, PP_RhoV, PP_radius;    /* PP_radius < 0: 0.25*ChLength */
    double noise_rho0, noise_amp;                          /* pp_noise init */
    uint64_t seed;
    double d2v16_c;                                        /* D2V16 lattice speed (1.2) */
    int uw;                                                /* the UW flux scheme (Allen-Cahn, periodic) with the
                                                              6-point (1), least-squares (2) or 4-point (3)
                                                              cell gradient; 0: CD */
    int nee;                                               /* 1: NEE walls instead of bounce-back */
} orc_inputs;

typedef struct orc_state orc_state;

orc_state *orc_create(const orc_inputs *in);
void orc_destroy(orc_state *s);
int orc_nq(const orc_state *s);
/* advance nsteps steps; nthreads <= 0 means all OpenMP threads */
void orc_step(orc_state *s, int nsteps, int nthreads);
long orc_steps_done(const orc_state *s);
/* copy a cell field [ny][nx]; names as in the reference dumps:
 * rho u v p phi phix phiy rhox rhoy fx fy prevphiu prevphiv psi tauf f<q> h<q> */
int orc_get(const orc_state *s, const char *name, double *out);
int orc_set(orc_state *s, const char *name, const double *in);
/* derived constant by name (dt, hDt, RT, Kp, aPhi, ...); NaN if unknown */
double orc_const(const orc_state *s, const char *name);
/* sums in cell order j-major: sum rho, sum phi */
void orc_sums(const orc_state *s, double *sum_rho, double *sum_phi);
/* the model's discrete velocities and |xi|^2 + eta^2 (D2V16: eta^2 on the first four) */
int orc_velocities(const orc_state *s, double *xi_u, double *xi_v, double *xi2);
/* D2V16 equilibrium (Macro16 x inverse moment matrix) at (rho, u, v); -1 for other models */
int orc_d2v16_equilibrium(const orc_state *s, double rho, double u, double v, double *eq);

#ifdef __cplusplus
}
#endif
#endif
