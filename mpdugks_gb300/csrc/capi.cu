// C ABI of libdugks_gpu.so (declared in include/dugks_gpu.h).
//
// Host side of the drop-in: derives the case constants with the reference's
// header formulas, allocates the resident device state, runs the reference's
// initialisation functions on the host, and drives the step kernels.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/dugks_gpu.h"
#include "dugks_device.cuh"

namespace dugks {
#define DUGKS_DECLARE_FP64(NS)                                                                                  \
    namespace NS {                                                                                              \
    void launch_fp64_step(const Params &P, const State &S, int do_msrc, int gin, int gout, cudaStream_t st,     \
                          int64_t *launches, cudaEvent_t *ev);                                                  \
    void launch_fp64_finalize(const Params &P, const State &S, int gin, cudaStream_t st, int64_t *launches);   \
    void launch_reduce(const Params &P, const double *rho, const double *phi, double *rho_last, double *partial, \
                       int nblocks, double *out4, int has_phi, cudaStream_t st, int64_t *launches);             \
    void launch_check_finite(const double *a, size_t n, int *flag, cudaStream_t st, int64_t *launches);         \
    }
DUGKS_DECLARE_FP64(exact)
DUGKS_DECLARE_FP64(fast)
}  // namespace dugks
#include "fp32_state.cuh"
#include "fp32_pp.cuh"
#include "trace.hpp"
namespace dugks {
namespace f32 {
cudaError_t launch_step32(const P32 &P, const S32 &S, int first, int gin, int gout, cudaStream_t st,
                          int64_t *launches, uint32_t step);
void launch_macros32(const P32 &P, const S32 &S, double *rho, double *u, double *v, double *p, double *phi,
                     int opitch, cudaStream_t st, int64_t *launches);
cudaError_t launch_step64f(const PR<double> &P, const SR<double> &S, int first, int gin, int gout,
                           cudaStream_t st, int64_t *launches, uint32_t step);
void launch_macros64f(const PR<double> &P, const SR<double> &S, double *rho, double *u, double *v, double *p,
                      double *phi, int opitch, cudaStream_t st, int64_t *launches);
cudaError_t launch_stream32(const P32 &P, const S32 &S, int first, int gin, int gout, cudaStream_t st,
                            int64_t *launches, uint32_t step, const void *tmap, int zin, int *err);
cudaError_t stream_tensor_map(void *map_out, float *base, int nx, int ny, int pitch, size_t qs);
cudaError_t launch_uw32(const P32 &P, const S32 &S, float *U, int first, cudaStream_t st, int64_t *launches);
cudaError_t launch_pp32_step(const PPP &P, const PPS &S, int do_msrc, cudaStream_t st, int64_t *launches,
                             uint32_t step);
cudaError_t launch_pp32_force(const PPP &P, const PPS &S, cudaStream_t st, int64_t *launches);
cudaError_t launch_pp32_stream(const PPP &P, const PPV &in, const PPV &out, float *Fx, float *Fy, double *p,
                               size_t qs, int do_msrc, cudaStream_t st, int64_t *launches);
cudaError_t launch_pp_g_from_f64(float *g, int pitch, const double *f, const double *rho, int nx, int ny, double e,
                                 cudaStream_t st, int64_t *launches);
template <typename R>
cudaError_t launch_plane_from_f64(R *dst, int dpitch, const double *src, int nx, int ny, double sub,
                                  cudaStream_t st, int64_t *launches);
template <typename R>
cudaError_t launch_phase_from_f64(R *g, R *phi, size_t qs, int pitch, const double *h, int nx, int ny,
                                  cudaStream_t st, int64_t *launches);
template <typename R>
void launch_out_forces(const PR<R> &P, const SR<R> &S, const double *phi, const double *rho, int opitch, int first,
                       double *tau, double *fx, double *fy, cudaStream_t st, int64_t *launches);
inline cudaError_t launch_stepX(const P32 &P, const S32 &S, int a, int b, int c, cudaStream_t st, int64_t *l,
                                uint32_t step) {
    return launch_step32(P, S, a, b, c, st, l, step);
}
inline cudaError_t launch_stepX(const PR<double> &P, const SR<double> &S, int a, int b, int c, cudaStream_t st,
                                int64_t *l, uint32_t step) {
    return launch_step64f(P, S, a, b, c, st, l, step);
}
inline void launch_macrosX(const P32 &P, const S32 &S, double *rho, double *u, double *v, double *p, double *phi,
                           int op, cudaStream_t st, int64_t *l) {
    launch_macros32(P, S, rho, u, v, p, phi, op, st, l);
}
inline void launch_macrosX(const PR<double> &P, const SR<double> &S, double *rho, double *u, double *v, double *p,
                           double *phi, int op, cudaStream_t st, int64_t *l) {
    launch_macros64f(P, S, rho, u, v, p, phi, op, st, l);
}
}  // namespace f32
using exact::launch_reduce;
using exact::launch_check_finite;
void build_d2v16_matrix(double c, double out[16][16]);
void derive_params(const dugks_case_t &cs, const dugks_grid_t &g, Params &P);
int host_init_state(const Params &P, const double iM[16][16], int kind, const double *params, int nparams,
                    uint64_t seed, std::vector<double> &f, std::vector<double> &h, std::vector<double> &aux);
void pp_rest_eq(const Params &P, const double iM[16][16], double rho, double *eq);
}  // namespace dugks

using namespace dugks;

struct dugks_handle {
    dugks_case_t cs;
    dugks_grid_t grid;
    Params P;
    State S;
    double iM[16][16];
    char *arena = nullptr;   // one device allocation for the whole state
    size_t arena_bytes = 0;
    double *rho_last = nullptr, *partial = nullptr, *out4 = nullptr;
    int *flag = nullptr;
    int nblocks = 0;
    int pending = 0;         // MacroSource / cell force of the last step not yet run
    int gcur = 0;            // ghost-phi buffer written by the last collision launch
    int64_t launches = 0;
    int64_t steps = 0;
    cudaStream_t last_stream = nullptr;
    std::string err;
    // fused deviation-form step (FP32 storage, or the same step in FP64)
    bool fp32 = false;        // any fused variant
    bool fused64 = false;     // the FP64 instance
    f32::P32 P32{};
    f32::S32 S32{};
    f32::PR<double> P64f{};
    f32::SR<double> S64f{};
    int first = 1;            // next step is the first after an upload
    // TMA staging of the streaming FP32 step: a tensor map over both state copies
    // (from tmap_base, the arena's first plane) and the error word of its staged loads
    CUtensorMap tmap{};
    bool has_tmap = false;
    const float *tmap_base = nullptr;
    int *kerr = nullptr;
    float *uw32 = nullptr;    // scratch planes of the FP32 UW step (f32::UW_PLANES)
    bool macros_fresh = false;
    double *out3 = nullptr;   // tau, Fx, Fy for output (allocated on first request)
    // FP32 storage of the pseudopotential models
    bool pp32 = false;
    f32::PPP PPc{};
    f32::PPS PPs{};
    int pp_pending = 0;       // the next collision computes the cell force from psi
    int init_kind = -1;       // the last dugks_gpu_init's kind and drop radius (drop L2 norm)
    double init_radius = 0.0;
    const double *pp_rho0 = nullptr;  // the density plane the step reads as created (checkpoint orientation)
    bool pp_stream = false;           // FP32 pseudopotential: the single-pass step (else three passes)
};

static std::string g_create_err;

namespace dugks {
// error text for entry points that have no handle (read by dugks_gpu_last_error(NULL, ...))
void set_global_error(const std::string &msg) { g_create_err = msg; }
}  // namespace dugks

using step_fn = void (*)(const Params &, const State &, int, int, int, cudaStream_t, int64_t *, cudaEvent_t *);
static step_fn step_launcher(const dugks_handle *h) {
    return h->cs.precision == DUGKS_FP64_FMA ? fast::launch_fp64_step : exact::launch_fp64_step;
}

static int fail(dugks_handle *h, int code, const std::string &msg) {
    if (h) h->err = msg;
    else g_create_err = msg;
    return code;
}

static int cuda_fail(dugks_handle *h, cudaError_t e, const char *what) {
    return fail(h, DUGKS_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// The device address of host memory the device can access in place (pinned and mapped:
// cudaHostAlloc, or registered with the mapped flag), else null.  On the GB300 such memory
// is read and written by kernels over NVLink-C2C, with no copy-engine staging.
static void *mapped_host(const void *p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// constants of the fused step: FP64 reference expressions, rounded once to R.
template <typename R>
static void derive_p32(const Params &P, f32::PR<R> &Q) {
    Q = f32::PR<R>{};
    Q.nx = P.nx; Q.ny = P.ny; Q.pitch = P.pitch; Q.walls = P.walls; Q.model = P.model; Q.gravity = P.gravity;
    Q.phi0 = (R)DUGKS_F32_PHI0; Q.p0 = R(1.0);
    Q.aPhi = (R)P.aPhi; Q.bPhi = (R)P.bPhi; Q.Kp = (R)P.Kp; Q.RT = (R)P.RT;
    Q.invRT = (R)(1.0 / P.RT); Q.hDt = (R)P.hDt; Q.dt = (R)P.dt; Q.Lambda0 = (R)P.Lambda0;
    Q.Beta = (R)P.Beta; Q.Kappa = (R)P.Kappa; Q.PhiL = (R)P.PhiL; Q.PhiV = (R)P.PhiV;
    Q.RhoL = (R)P.RhoL; Q.Gy = (R)P.Gy;
    Q.inv_12dx = (R)(1.0 / (P._2dx * 6)); Q.inv_12dy = (R)(1.0 / (P._2dy * 6));
    Q.inv_6dd = (R)(1.0 / (6 * P.MinL * P.MinL));
    Q.inv_wI_dphi = (R)(1.0 / (P.wI * (P.PhiL - P.PhiV)));
    Q.inv_RTdt = (R)(1.0 / (P.RT * P.dt));
    // after the first step tau = Mu/(rho RT) = Tau0 for both Allen-Cahn models (nu_L = nu_V = nu0)
    const double tau = P.Tau0;
    const double aBP = (2.0 * tau - P.hDt) / (2.0 * tau + P.dt), ah = 2.0 * tau / (2.0 * tau + P.hDt);
    Q.tauf = (R)tau; Q.aBP_f = (R)aBP; Q.ah_f = (R)ah;
    Q.h_aBP = (R)P.h_aBP; Q.h_bBP = (R)P.h_bBP; Q.h_cBP = (R)P.h_cBP;
    Q.h_ah = (R)P.h_ah; Q.h_bh = (R)P.h_bh; Q.h_ch = (R)P.h_ch;
    Q.r_2dy = (R)P.r_2dy; Q.r_ndx = (R)P.r_ndx; Q.r_n2dx = (R)P.r_n2dx; Q.r_ndy = (R)P.r_ndy;
    Q.aTP = (R)P.aTP; Q.bTP = (R)P.bTP; Q.dtV = (R)P.dtV;
    Q.nee = P.nee;
    Q.uw_grad = P.uw_grad;
    Q.hneq = (R)(2.0 * P.TauMass / (2.0 * P.TauMass + P.dt));
}

// rest equilibria the deviations are taken from
static double f_rest(const Params &P, int q) {
    const double p0 = 1.0;
    if (P.model == AC) return P.omega[q] * p0 / P.RT - (q == 0 ? p0 / P.RT : 0.0);
    return P.omega[q] * p0;
}

constexpr int REDUCE_BLOCKS = 152 * 4;

// device bytes of one case of the fused step with storage type of rsize bytes
static size_t fused_arena_bytes(const Params &P, size_t rsize) {
    const size_t rowf = (size_t)P.pitch * rsize;
    const size_t cellf = align256(rowf * P.ny);
    const size_t celld = align256((size_t)P.pitch * sizeof(double) * P.ny);
    return 2 * f32::PL_N * cellf + f32::I_N * cellf + align256(f32::GPHI_ROWS * rowf) +
           6 * celld /* rho u v p phi + rho_last */ + align256(sizeof(double) * 4 * REDUCE_BLOCKS) + 512 +
           (P.uw ? f32::UW_PLANES * cellf : 0) /* the UW step's scratch */;
}

// device bytes of one case of the multi-kernel FP64 step
static size_t fp64_arena_bytes(const Params &P) {
    const size_t rowb = (size_t)P.pitch * sizeof(double);
    const size_t cellb = align256(rowb * P.ny), ycellb = align256(rowb * (P.ny + 1));
    const int Q = P.Q;
    const bool pp = !(P.model == AC || P.model == HCZ);
    size_t total = 0;
    total += 2 * Q * cellb;                       // f, h (h unused by PP but kept simple)
    total += 2 * Q * cellb;                       // bf, bh
    total += 2 * Q * cellb + 2 * Q * ycellb;      // x/y face fluxes
    total += NFIELDS * cellb;                     // macro fields
    total += align256(4 * rowb);                  // ghost phi rows
    if (pp) total += 14 * cellb + 2 * Q * cellb;  // pseudopotential face state + face BhDt
    if (P.nee) total += align256(sizeof(double) * 8 * Q * P.pitch);  // NEE wall-row equilibria/sources
    if (P.uw)                                     // UW cell gradients of f and h, low-side boundary fluxes
        total += 4 * Q * cellb + 2 * align256(sizeof(double) * Q * P.ny) + 2 * Q * rowb;
    total += cellb;                               // rho_last
    total += align256(sizeof(double) * 4 * REDUCE_BLOCKS) + 256 + 256;
    if (P.model == PP16) total += align256(sizeof(double) * 256);  // the case's D2V16 inverse moment matrix
    return total;
}

static cudaError_t to_dev(const dugks_handle *h, double *d, const double *src, int rows = -1);

// device bytes of one FP32 pseudopotential case
static size_t pp32_arena_bytes(const Params &P) {
    const size_t cf = align256((size_t)P.pitch * P.ny * sizeof(float));
    const size_t cd = align256((size_t)P.pitch * P.ny * sizeof(double));
    // multi-pass state and scratch, plus the single-pass step's second copy (Q + 7 float
    // planes, U and V)
    return (7 * (size_t)P.Q + 28) * cf + 9 * cd + align256(sizeof(double) * 4 * REDUCE_BLOCKS) + 512;
}

// after a step of the FP32 pseudopotential path: the density the update wrote (and, for
// the single-pass step, the whole copy it wrote) becomes the state
static void pp32_swap(dugks_handle *h) {
    std::swap(h->PPs.rho, h->PPs.rho_o);
    if (h->pp_stream) f32::pp_swap_copies(h->PPs);
    h->S.fld[F_RHO] = h->PPs.rho;
    h->S.fld[F_U] = h->PPs.U;
    h->S.fld[F_V] = h->PPs.V;
}

// a double as the unevaluated float sum hi + lo (about 48 significant bits)
static void split_ff(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// The D2V16 equilibria (pp_deq, fp32_pp.cuh; d2v16_eq, fp64_step.cuh) skip the inverse
// moment matrix's structural zeros, and the FP32 and FP64-FMA ones evaluate it by
// opposite-direction pairs: check that this case's matrix has that form (opposite rows
// equal in the even moments' entries, negated in the odd ones; zeros where d2v16_entry
// says), so a change of the table cannot go unnoticed.
static bool d2v16_matrix_has_pair_form(const double (&iM)[16][16]) {
    for (int j = 0; j < 16; ++j) {
        const int jo = d2v16_opp(j);
        for (int k = 0; k < 16; ++k) {
            if (!d2v16_entry(j, k) && (iM[j][k] != 0.0 || iM[jo][k] != 0.0)) return false;
            if (iM[jo][k] != (d2v16_odd_moment(k) ? -iM[j][k] : iM[j][k])) return false;
        }
    }
    return true;
}

static int create_pp32(dugks_handle *h, dugks_handle_t **out) {
    Params &P = h->P;
    h->pp32 = true;
    // the three-pass step; DUGKS_PP_PASSES=1 in the environment selects the single-pass
    // streaming step (grids of at least 32 columns and 8 rows).  The two give the same
    // results; on the GB300 the three-pass form is 1.75x faster (the single pass holds a row
    // pipeline of 16 distributions per lane: ~10 warps per SM, latency-bound)
    const char *passes = std::getenv("DUGKS_PP_PASSES");
    h->pp_stream = P.nx >= 32 && P.ny >= 8 && passes && std::atoi(passes) == 1;
    h->nblocks = REDUCE_BLOCKS;
    const size_t cf = align256((size_t)P.pitch * P.ny * sizeof(float));
    const size_t cd = align256((size_t)P.pitch * P.ny * sizeof(double));
    const size_t total = pp32_arena_bytes(P);
    cudaError_t e = cudaMalloc(&h->arena, total);
    if (e != cudaSuccess) {
        delete h;
        return fail(nullptr, e == cudaErrorMemoryAllocation ? DUGKS_ENOMEM : DUGKS_ECUDA,
                    std::string("cudaMalloc of device state failed: ") + cudaGetErrorString(e));
    }
    h->arena_bytes = total;
    cudaMemsetAsync(h->arena, 0, total, nullptr);
    char *cur = h->arena;
    auto tf = [&](size_t n) { float *p = reinterpret_cast<float *>(cur); cur += n * cf; return p; };
    auto td = [&]() { double *p = reinterpret_cast<double *>(cur); cur += cd; return p; };
    f32::PPS &S = h->PPs;
    const int Q = P.Q;
    S.qs = cf / sizeof(float);
    S.df = tf(Q);
    S.bf = tf(Q);
    S.xb = tf(Q);
    S.yb = tf(Q);
    S.xfl = tf(Q);
    S.yfl = tf(Q);
    float **scal[] = {&S.xr, &S.yr, &S.xu, &S.yu, &S.xv, &S.yv, &S.xg, &S.yg, &S.xps, &S.yps,
                      &S.xFx, &S.xFy, &S.yFx, &S.yFy, &S.psi, &S.scg, &S.Fx, &S.Fy,
                      &S.psil, &S.xpsl, &S.ypsl};
    for (auto p : scal) *p = tf(1);
    S.alt.g = tf(Q);
    float **alt[] = {&S.alt.psi, &S.alt.psil, &S.alt.scg, &S.alt.xFx, &S.alt.xFy, &S.alt.yFx, &S.alt.yFy};
    for (auto p : alt) *p = tf(1);
    S.alt.U = td();
    S.alt.V = td();
    S.alt.rho = nullptr;
    S.rho = td();
    S.rho_o = td();
    h->pp_rho0 = S.rho;
    S.p = td();
    S.U = td();
    S.V = td();
    h->S.fld[F_RHO] = S.rho;
    h->S.fld[F_P] = S.p;
    h->S.fld[F_U] = S.U;
    h->S.fld[F_V] = S.V;
    h->S.fld[F_PHI] = td();  // no phase field: zeros for the reductions and downloads
    h->rho_last = td();
    h->partial = reinterpret_cast<double *>(cur);
    cur += align256(sizeof(double) * 4 * REDUCE_BLOCKS);
    h->out4 = reinterpret_cast<double *>(cur);
    cur += 256;
    h->flag = reinterpret_cast<int *>(cur);
    // constants
    f32::PPP &C = h->PPc;
    C.nx = P.nx;
    C.ny = P.ny;
    C.pitch = P.pitch;
    C.model = P.model;
    C.Q = Q;
    C.hDt = (float)P.hDt;
    C.dt = (float)P.dt;
    C.RT = (float)P.RT;
    C.invRT = (float)(1.0 / P.RT);
    C.Lambda0 = (float)P.Lambda0;
    C.Tau0 = (float)P.Tau0;
    C.aTP = (float)P.aTP;
    C.bTP = (float)P.bTP;
    C.dtV = (float)P.dtV;
    C.r_2dy = (float)P.r_2dy;
    C.r_ndx = (float)P.r_ndx;
    C.r_n2dx = (float)P.r_n2dx;
    C.r_ndy = (float)P.r_ndy;
    C.inv_6_2dx = (float)(1.0 / (P._2dx * 6));
    C.inv_6_2dy = (float)(1.0 / (P._2dy * 6));
    C.R0 = P.R0;
    C.T_CS = P.T_CS;
    C.aCS = P.aCS;
    C.RTd = P.RT;
    split_ff(P.R0 * P.T_CS, C.rtcs_hi, C.rtcs_lo);
    split_ff(P.aCS, C.acs_hi, C.acs_lo);
    split_ff(P.RT, C.rt_hi, C.rt_lo);
    split_ff(P.c16, C.lat_hi, C.lat_lo);
    for (int q = 0; q < Q; ++q) {
        C.xi_u[q] = (float)P.xi_u[q];
        C.xi_v[q] = (float)P.xi_v[q];
    }
    for (int q = 0; q < 9; ++q) C.w9[q] = (float)P.omega[q];
    {   // the rest equilibrium per unit density, e_q = eq_q(1, 0, 0)
        double rest[16];
        pp_rest_eq(P, h->iM, 1.0, rest);
        for (int q = 0; q < Q; ++q) C.erest[q] = (float)rest[q];
    }
    // this case's inverse moment matrix in FP32 (zeros for D2Q9PP)
    for (int j = 0; j < 16; ++j)
        for (int k = 0; k < 16; ++k) C.iM16[j][k] = P.model == PP16 ? (float)h->iM[j][k] : 0.f;
    e = cudaStreamSynchronize(nullptr);
    if (e != cudaSuccess) {
        cudaFree(h->arena);
        delete h;
        return fail(nullptr, DUGKS_ECUDA, std::string("device setup failed: ") + cudaGetErrorString(e));
    }
    *out = h;
    return DUGKS_OK;
}

// FP64 [Q][ny][nx] state -> deviations from the rest equilibrium at the mean density
static int upload_pp32(dugks_handle *h, const double *f, const double *aux) {
    const Params &P = h->P;
    const int nx = P.nx, ny = P.ny;
    const size_t n = (size_t)nx * ny;
    cudaStream_t st = h->last_stream;
    f32::PPP &C = h->PPc;
    f32::PPS &S = h->PPs;
    cudaError_t e;
    // the FP64 planes of the state as uploaded (the density first: the remainders are
    // taken against it); face forces and psi restart
    const int fid[4] = {F_RHO, F_U, F_V, F_P};
    for (int k : fid)
        if ((e = to_dev(h, h->S.fld[k], aux + (size_t)k * n)) != cudaSuccess) return cuda_fail(h, e, "upload");
    double *stage = nullptr;
    e = cudaMalloc(&stage, n * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(h, e, "upload staging");
    // g_q = f_q - e_q rho
    for (int q = 0; q < P.Q && e == cudaSuccess; ++q) {
        e = cudaMemcpyAsync(stage, f + (size_t)q * n, n * sizeof(double), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = f32::launch_pp_g_from_f64(S.df + (size_t)q * S.qs, P.pitch, stage, S.rho, nx, ny, (double)C.erest[q],
                                          st, &h->launches);
    }
    auto put = [&](float *dst, const double *src) -> cudaError_t {
        cudaError_t r = cudaMemcpyAsync(stage, src, n * sizeof(double), cudaMemcpyHostToDevice, st);
        if (r != cudaSuccess) return r;
        return f32::launch_plane_from_f64<float>(dst, P.pitch, stage, nx, ny, 0.0, st, &h->launches);
    };
    if (e == cudaSuccess) e = put(S.Fx, aux + (size_t)F_FX * n);
    if (e == cudaSuccess) e = put(S.Fy, aux + (size_t)F_FY * n);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(stage);
    if (e != cudaSuccess) return cuda_fail(h, e, "upload");
    float *zero[] = {S.xFx, S.xFy, S.yFx, S.yFy, S.psi, S.scg, S.psil, S.xpsl, S.ypsl};
    for (auto z : zero) cudaMemsetAsync(z, 0, S.qs * sizeof(float), st);
    cudaMemsetAsync(h->rho_last, 0, (size_t)P.pitch * ny * sizeof(double), st);
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(h, e, "upload");
    h->pp_pending = 0;
    h->steps = 0;
    return DUGKS_OK;
}

// an FP32 plane of the pseudopotential state as FP64 [ny][nx]
static int pp32_plane_to_host(dugks_handle *h, const float *d, double *out) {
    const Params &P = h->P;
    std::vector<float> tmp((size_t)P.nx * P.ny);
    cudaError_t e = cudaMemcpy2DAsync(tmp.data(), (size_t)P.nx * sizeof(float), d, (size_t)P.pitch * sizeof(float),
                                      (size_t)P.nx * sizeof(float), P.ny, cudaMemcpyDeviceToHost, h->last_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->last_stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "download field");
    for (size_t k = 0; k < tmp.size(); ++k) out[k] = tmp[k];
    return DUGKS_OK;
}

template <typename R>
static int create_fused(dugks_handle *h, dugks_handle_t **out, f32::PR<R> &PQ, f32::SR<R> &S) {
    Params &P = h->P;
    h->fp32 = true;
    derive_p32<R>(P, PQ);
    const size_t rowf = (size_t)P.pitch * sizeof(R);
    const size_t cellf = align256(rowf * P.ny);
    const size_t rowd = (size_t)P.pitch * sizeof(double);
    const size_t celld = align256(rowd * P.ny);
    h->nblocks = REDUCE_BLOCKS;
    const size_t total = fused_arena_bytes(P, sizeof(R));
    cudaError_t e = cudaMalloc(&h->arena, total);
    if (e != cudaSuccess) {
        delete h;
        return fail(nullptr, e == cudaErrorMemoryAllocation ? DUGKS_ENOMEM : DUGKS_ECUDA,
                    std::string("cudaMalloc of device state failed: ") + cudaGetErrorString(e));
    }
    h->arena_bytes = total;
    cudaMemsetAsync(h->arena, 0, total, nullptr);
    char *cur = h->arena;
    auto takef = [&](size_t b) { R *p = reinterpret_cast<R *>(cur); cur += b; return p; };
    auto taked = [&](size_t b) { double *p = reinterpret_cast<double *>(cur); cur += b; return p; };
    S.qs = cellf / sizeof(R);
    // two state copies of PL_N planes each (f, g, the phi pair, aux; fp32_state.cuh)
    R *copy0 = takef(f32::PL_N * cellf), *copy1 = takef(f32::PL_N * cellf);
    f32::set_copy(copy0, S.qs, S.df, S.dg, S.phi, S.aux);
    f32::set_copy(copy1, S.qs, S.odf, S.odg, S.ophi, S.oaux);
    S.init = takef(f32::I_N * cellf);
    S.gphi = takef(align256(f32::GPHI_ROWS * rowf));
    const int fids[5] = {F_RHO, F_U, F_V, F_P, F_PHI};
    for (int k : fids) h->S.fld[k] = taked(celld);
    h->rho_last = taked(celld);
    h->partial = taked(align256(sizeof(double) * 4 * h->nblocks));
    h->out4 = taked(256);
    h->flag = reinterpret_cast<int *>(taked(256));
    if (P.uw) h->uw32 = reinterpret_cast<float *>(takef(f32::UW_PLANES * cellf));
    e = cudaStreamSynchronize(nullptr);  // the clear above (legacy stream; leaves non-blocking streams running)
    if (e != cudaSuccess) {
        cudaFree(h->arena);
        delete h;
        return fail(nullptr, DUGKS_ECUDA, std::string("device setup failed: ") + cudaGetErrorString(e));
    }
    *out = h;
    return DUGKS_OK;
}

static int create_fp32(dugks_handle *h, dugks_handle_t **out) {
    if (h->cs.precision == DUGKS_FP64_FUSED) {
        h->fused64 = true;
        return create_fused<double>(h, out, h->P64f, h->S64f);
    }
    int rc = create_fused<float>(h, out, h->P32, h->S32);
    if (rc) return rc;
    // the streaming step's stage loads go through TMA where a tensor map can describe
    // the state (any grid of at least 32 columns); otherwise they are per-lane copies
    h->kerr = h->flag + 32;  // a spare word of the zeroed 256-byte flag block
    if (f32::stream_tensor_map(&h->tmap, h->S32.df, h->P.nx, h->P.ny, h->P.pitch, h->S32.qs) == cudaSuccess) {
        h->has_tmap = true;
        h->tmap_base = h->S32.df;
    }
    return DUGKS_OK;
}

// FP64 [Q][ny][nx] state -> deviations and first-step planes on the device.
// Each FP64 plane is copied as-is into a device staging plane and converted there.  The
// host-to-device copies run on a stream of their own through two staging planes (two of
// the FP64 output fields, which an upload invalidates anyway), so the copy of a plane
// overlaps the conversion of the one before on the handle's stream; a host plane that
// feeds several device planes (the forces and density gradients: first-step inputs and
// the previous MacroSource) is copied once.
template <typename R>
static int upload_fused(dugks_handle *h, f32::SR<R> &S, const double *f, const double *hd, const double *aux) {
    const Params &P = h->P;
    const int nx = P.nx, ny = P.ny;
    const size_t n = (size_t)nx * ny, bytes = n * sizeof(double);
    cudaStream_t st = h->last_stream, cs = nullptr;
    cudaEvent_t ev[5] = {};  // staging plane copied (2), staging plane consumed (2), h copied
    struct Cleanup {
        cudaStream_t &cs;
        cudaEvent_t (&ev)[5];
        ~Cleanup() {
            if (cs) cudaStreamSynchronize(cs);
            for (auto &x : ev)
                if (x) cudaEventDestroy(x);
            if (cs) cudaStreamDestroy(cs);
        }
    } cleanup{cs, ev};
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    for (auto &x : ev)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(h, e, "upload streams");
    double *stage[2] = {h->S.fld[F_RHO], h->S.fld[F_U]};
    // host arrays the device can read in place (pinned and mapped): the conversions read
    // them directly (measured on the 8192^2 state, 18 GB: 92 ms against 82 ms through the
    // copy engines on an idle GPU, but 138-166 ms against 210-861 ms right after a run of
    // steps, when the copy-engine path slowed down and this one much less)
    const double *fm = static_cast<const double *>(mapped_host(f));
    const double *hm = hd ? static_cast<const double *>(mapped_host(hd)) : nullptr;
    const double *am = static_cast<const double *>(mapped_host(aux));
    struct Dst {
        R *p;
        double sub;
    };
    int job = 0;
    auto put = [&](const double *src, const Dst *dsts, int nd, const double *dsrc) -> cudaError_t {
        if (dsrc) {
            cudaError_t r = cudaSuccess;
            for (int k = 0; k < nd && r == cudaSuccess; ++k)
                r = f32::launch_plane_from_f64<R>(dsts[k].p, P.pitch, dsrc, nx, ny, dsts[k].sub, st, &h->launches);
            return r;
        }
        const int b = job++ & 1;
        cudaError_t r = job > 2 ? cudaStreamWaitEvent(cs, ev[2 + b], 0) : cudaSuccess;
        if (r == cudaSuccess) r = cudaMemcpyAsync(stage[b], src, bytes, cudaMemcpyHostToDevice, cs);
        if (r == cudaSuccess) r = cudaEventRecord(ev[b], cs);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(st, ev[b], 0);
        for (int k = 0; k < nd && r == cudaSuccess; ++k)
            r = f32::launch_plane_from_f64<R>(dsts[k].p, P.pitch, stage[b], nx, ny, dsts[k].sub, st, &h->launches);
        if (r == cudaSuccess) r = cudaEventRecord(ev[2 + b], st);
        return r;
    };
    for (int q = 0; q < 9; ++q) {
        const Dst d = {S.df + q * S.qs, f_rest(P, q)};
        if ((e = put(f + q * n, &d, 1, fm ? fm + q * n : nullptr)) != cudaSuccess) return cuda_fail(h, e, "upload f");
    }
    // the phase field: the nine FP64 h planes go to the copy the next step writes (free
    // until then: 9 n doubles fit in its PL_N planes), then phi = sum_q h_q as a pair and
    // g_q = h_q - w_q phi into the copy it reads
    {
        const double *hst = hm;
        if (!hst) {
            double *hs = reinterpret_cast<double *>(S.odf);
            e = cudaMemcpyAsync(hs, hd, 9 * bytes, cudaMemcpyHostToDevice, cs);
            if (e == cudaSuccess) e = cudaEventRecord(ev[4], cs);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev[4], 0);
            hst = hs;
        }
        if (e == cudaSuccess) e = f32::launch_phase_from_f64<R>(S.dg, S.phi, S.qs, P.pitch, hst, nx, ny, st, &h->launches);
        if (e != cudaSuccess) return cuda_fail(h, e, "upload h");
    }
    // first-step inputs (init planes) and the previous MacroSource outputs (aux planes)
    const size_t qs = S.qs;
    R *I = S.init, *A = S.aux;
    struct Plane {
        int field, nd;
        Dst d[2];
    };
    const Plane planes[] = {
        {F_PHI, 1, {{I + f32::I_DPHI * qs, DUGKS_F32_PHI0}, {}}},
        {F_RHO, 1, {{I + f32::I_RHO * qs, 0.0}, {}}},
        {F_U, 1, {{I + f32::I_U * qs, 0.0}, {}}},
        {F_V, 1, {{I + f32::I_V * qs, 0.0}, {}}},
        {F_P, 1, {{I + f32::I_DP * qs, 1.0}, {}}},
        {F_TAU, 1, {{I + f32::I_TAU * qs, 0.0}, {}}},
        {F_PHIX, 1, {{I + f32::I_SRCX * qs, 0.0}, {}}},
        {F_PHIY, 1, {{I + f32::I_SRCY * qs, 0.0}, {}}},
        {F_RHOX, 2, {{I + f32::I_RHOX * qs, 0.0}, {A + f32::A_RHOX * qs, 0.0}}},
        {F_RHOY, 2, {{I + f32::I_RHOY * qs, 0.0}, {A + f32::A_RHOY * qs, 0.0}}},
        {F_FX, 2, {{I + f32::I_FX * qs, 0.0}, {A + f32::A_FX * qs, 0.0}}},
        {F_FY, 2, {{I + f32::I_FY * qs, 0.0}, {A + f32::A_FY * qs, 0.0}}},
        {F_PPU, 1, {{A + f32::A_PPU * qs, 0.0}, {}}},
        {F_PPV, 1, {{A + f32::A_PPV * qs, 0.0}, {}}},
    };
    for (const Plane &pl : planes)
        if ((e = put(aux + (size_t)pl.field * n, pl.d, pl.nd, am ? am + (size_t)pl.field * n : nullptr)) != cudaSuccess)
            return cuda_fail(h, e, "upload init");
    if ((e = cudaMemsetAsync(h->rho_last, 0, (size_t)P.pitch * ny * sizeof(double), st)) != cudaSuccess)
        return cuda_fail(h, e, "upload");
    // the handle's stream waited for every copy before converting it
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(h, e, "upload");
    h->first = 1;
    h->gcur = 0;
    h->steps = 0;
    h->macros_fresh = false;
    return DUGKS_OK;
}

static int upload_fp32(dugks_handle *h, const double *f, const double *hd, const double *aux) {
    return h->fused64 ? upload_fused<double>(h, h->S64f, f, hd, aux) : upload_fused<float>(h, h->S32, f, hd, aux);
}

static int macros_fp32(dugks_handle *h) {
    if (h->macros_fresh) return DUGKS_OK;
    if (h->fused64)
        f32::launch_macrosX(h->P64f, h->S64f, h->S.fld[F_RHO], h->S.fld[F_U], h->S.fld[F_V], h->S.fld[F_P],
                            h->S.fld[F_PHI], h->P.pitch, h->last_stream, &h->launches);
    else
        f32::launch_macrosX(h->P32, h->S32, h->S.fld[F_RHO], h->S.fld[F_U], h->S.fld[F_V], h->S.fld[F_P],
                            h->S.fld[F_PHI], h->P.pitch, h->last_stream, &h->launches);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(h, e, "macros launch");
    h->macros_fresh = true;
    return DUGKS_OK;
}

// the streaming step's staged loads all completed (read after a synchronisation of
// the handle's stream); DUGKS_ETIMEOUT once one did not
static int stage_loads_ok(dugks_handle *h) {
    if (!h->kerr) return DUGKS_OK;
    int v = 0;  // on the handle's stream (the callers have just synchronised it)
    cudaError_t e = cudaMemcpyAsync(&v, h->kerr, sizeof v, cudaMemcpyDeviceToHost, h->last_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->last_stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "stage-load status");
    return v ? fail(h, DUGKS_ETIMEOUT, "a TMA stage load of the streaming step did not complete") : DUGKS_OK;
}

extern "C" int dugks_gpu_create(const dugks_case_t *c, const dugks_grid_t *g, dugks_handle_t **out) {
    if (!c || !g || !out) return fail(nullptr, DUGKS_EINVAL, "null argument");
    *out = nullptr;
    if (g->nx < 3 || g->ny < 3) return fail(nullptr, DUGKS_EINVAL, "nx and ny must be >= 3");
    if ((long long)g->nx * g->ny > (1LL << 31)) return fail(nullptr, DUGKS_EINVAL, "grid too large");
    if (c->model < DUGKS_MODEL_AC || c->model > DUGKS_MODEL_PP16)
        return fail(nullptr, DUGKS_EINVAL, "unknown model");
    if ((c->model == DUGKS_MODEL_PP9 || c->model == DUGKS_MODEL_PP16) && g->y_walls)
        return fail(nullptr, DUGKS_EINVAL, "pseudopotential models are periodic only (faceFaces need no walls)");
    if (c->precision < DUGKS_FP64 || c->precision > DUGKS_FP64_FUSED)
        return fail(nullptr, DUGKS_EINVAL, "unknown precision");
    if (c->precision == DUGKS_FP64_FUSED && !(c->model == DUGKS_MODEL_AC || c->model == DUGKS_MODEL_HCZ))
        return fail(nullptr, DUGKS_EINVAL, "the fused deviation-form step supports the Allen-Cahn models (AC, HCZ)");
    if (c->flux_scheme < DUGKS_FLUX_CD || c->flux_scheme > DUGKS_FLUX_UW_4P)
        return fail(nullptr, DUGKS_EINVAL, "unknown flux scheme");
    if (c->wall_scheme != DUGKS_WALL_BB && c->wall_scheme != DUGKS_WALL_NEE)
        return fail(nullptr, DUGKS_EINVAL, "unknown wall scheme");
    if (c->wall_scheme == DUGKS_WALL_NEE &&
        (!(c->precision == DUGKS_FP64 || c->precision == DUGKS_FP64_FMA || c->precision == DUGKS_FP32_DEV) ||
         !(c->model == DUGKS_MODEL_AC || c->model == DUGKS_MODEL_HCZ)))
        return fail(nullptr, DUGKS_EINVAL,
                    "NEE walls run with DUGKS_FP64 / DUGKS_FP64_FMA / DUGKS_FP32_DEV and the Allen-Cahn models");
    if (c->wall_scheme == DUGKS_WALL_NEE && c->precision == DUGKS_FP32_DEV && g->y_walls && g->ny < 8)
        return fail(nullptr, DUGKS_EINVAL, "NEE walls in FP32 storage need at least 8 rows (the streaming step)");
    if (c->flux_scheme != DUGKS_FLUX_CD &&
        (!(c->precision == DUGKS_FP64 || c->precision == DUGKS_FP64_FMA || c->precision == DUGKS_FP32_DEV) ||
         !(c->model == DUGKS_MODEL_AC || c->model == DUGKS_MODEL_HCZ) || g->y_walls))
        return fail(nullptr, DUGKS_EINVAL,
                    "the UW flux scheme runs with DUGKS_FP64 / DUGKS_FP64_FMA / DUGKS_FP32_DEV, the Allen-Cahn models "
                    "and periodic y (the reference's UW reads unwritten gradients of its wall shadow cells)");
    dugks_handle *h = new (std::nothrow) dugks_handle();
    if (!h) return fail(nullptr, DUGKS_ENOMEM, "host allocation failed");
    h->cs = *c;
    h->grid = *g;
    derive_params(*c, *g, h->P);
    Params &P = h->P;
    if (P.model == PP16) build_d2v16_matrix(P.c16, h->iM);
    if (P.model == PP16 && !d2v16_matrix_has_pair_form(h->iM)) {
        delete h;
        return fail(nullptr, DUGKS_EINVAL, "D2V16 inverse moment matrix without the opposite-pair form the step assumes");
    }
    if (c->precision == DUGKS_FP32_DEV && (P.model == PP9 || P.model == PP16)) return create_pp32(h, out);
    if (c->precision == DUGKS_FP32_DEV || c->precision == DUGKS_FP64_FUSED) return create_fp32(h, out);
    // ---- carve the arena
    const size_t rowb = (size_t)P.pitch * sizeof(double);
    const size_t cellb = align256(rowb * P.ny), ycellb = align256(rowb * (P.ny + 1));
    const int Q = P.Q;
    const bool pp = !(P.model == AC || P.model == HCZ);
    h->nblocks = REDUCE_BLOCKS;
    const size_t total = fp64_arena_bytes(P);
    cudaError_t e = cudaMalloc(&h->arena, total);
    if (e != cudaSuccess) {
        delete h;
        return fail(nullptr, e == cudaErrorMemoryAllocation ? DUGKS_ENOMEM : DUGKS_ECUDA,
                    std::string("cudaMalloc of device state failed: ") + cudaGetErrorString(e));
    }
    h->arena_bytes = total;
    e = cudaMemset(h->arena, 0, total);
    if (e != cudaSuccess) {
        cudaFree(h->arena);
        delete h;
        return fail(nullptr, DUGKS_ECUDA, std::string("cudaMemset failed: ") + cudaGetErrorString(e));
    }
    char *cur = h->arena;
    auto take = [&](size_t b) { double *p = reinterpret_cast<double *>(cur); cur += b; return p; };
    State &S = h->S;
    // velocity planes of one array are cellb / ycellb bytes apart
    S.qs = cellb / sizeof(double);
    S.qsy = ycellb / sizeof(double);
    S.f = take(Q * cellb);
    S.h = take(Q * cellb);
    S.bf = take(Q * cellb);
    S.bh = take(Q * cellb);
    S.xff = take(Q * cellb);
    S.xfh = take(Q * cellb);
    S.yff = take(Q * ycellb);
    S.yfh = take(Q * ycellb);
    for (int k = 0; k < NFIELDS; ++k) S.fld[k] = take(cellb);
    S.gphi = take(align256(4 * rowb));
    if (pp) {
        double **pf[] = {&S.xfFx, &S.xfFy, &S.yfFx, &S.yfFy, &S.xpsi, &S.ypsi, &S.xscg,
                         &S.yscg, &S.xrho, &S.yrho, &S.xu, &S.yu, &S.xv, &S.yv};
        for (auto p : pf) *p = take(cellb);
        S.xbf = take(Q * cellb);
        S.ybf = take(Q * cellb);
    }
    if (P.nee) S.weq = take(align256(sizeof(double) * 8 * Q * P.pitch));
    if (P.uw) {
        S.gfx = take(Q * cellb);
        S.gfy = take(Q * cellb);
        S.ghx = take(Q * cellb);
        S.ghy = take(Q * cellb);
        S.xlo_f = take(align256(sizeof(double) * Q * P.ny));
        S.xlo_h = take(align256(sizeof(double) * Q * P.ny));
        S.ylo_f = take(Q * rowb);
        S.ylo_h = take(Q * rowb);
    }
    h->rho_last = take(cellb);
    h->partial = take(align256(sizeof(double) * 4 * h->nblocks));
    h->out4 = take(256);
    h->flag = reinterpret_cast<int *>(take(256));
    P.iM16 = nullptr;
    if (P.model == PP16) {
        double *dm = take(align256(sizeof(double) * 256));
        e = cudaMemcpy(dm, &h->iM[0][0], sizeof(double) * 256, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(h->arena);
            delete h;
            return fail(nullptr, DUGKS_ECUDA, std::string("device setup failed: ") + cudaGetErrorString(e));
        }
        P.iM16 = dm;
    }
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        cudaFree(h->arena);
        delete h;
        return fail(nullptr, DUGKS_ECUDA, std::string("device setup failed: ") + cudaGetErrorString(e));
    }
    *out = h;
    return DUGKS_OK;
}

extern "C" int dugks_gpu_nq(const dugks_handle_t *h) { return h ? h->P.Q : 0; }

// host [ny][nx] <-> device [ny][pitch]
static cudaError_t to_dev(const dugks_handle *h, double *d, const double *src, int rows) {
    const Params &P = h->P;
    return cudaMemcpy2D(d, (size_t)P.pitch * sizeof(double), src, (size_t)P.nx * sizeof(double),
                        (size_t)P.nx * sizeof(double), rows < 0 ? P.ny : rows, cudaMemcpyHostToDevice);
}
static cudaError_t to_host(const dugks_handle *h, double *dst, const double *d) {
    const Params &P = h->P;
    return cudaMemcpy2D(dst, (size_t)P.nx * sizeof(double), d, (size_t)P.pitch * sizeof(double),
                        (size_t)P.nx * sizeof(double), P.ny, cudaMemcpyDeviceToHost);
}

static int sync_last(dugks_handle *h) {
    cudaError_t e = cudaStreamSynchronize(h->last_stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "stream synchronise");
    return DUGKS_OK;
}

extern "C" int dugks_gpu_upload(dugks_handle_t *h, const double *f, const double *hd, const double *aux) {
    if (!h || !f || !aux) return fail(h, DUGKS_EINVAL, "null argument");
    int rc = sync_last(h);
    if (rc) return rc;
    const Params &P = h->P;
    const size_t n = (size_t)P.nx * P.ny;
    const bool hasH = (P.model == AC || P.model == HCZ);
    if (hasH && !hd) return fail(h, DUGKS_EINVAL, "Allen-Cahn models need the h distribution");
    if (h->fp32) return upload_fp32(h, f, hd, aux);
    if (h->pp32) return upload_pp32(h, f, aux);
    cudaError_t e;
    for (int q = 0; q < P.Q; ++q) {
        if ((e = to_dev(h, h->S.f + q * h->S.qs, f + q * n)) != cudaSuccess) return cuda_fail(h, e, "upload f");
        if (hasH && (e = to_dev(h, h->S.h + q * h->S.qs, hd + q * n)) != cudaSuccess)
            return cuda_fail(h, e, "upload h");
    }
    for (int k = 0; k < NFIELDS; ++k)
        if ((e = to_dev(h, h->S.fld[k], aux + k * n)) != cudaSuccess) return cuda_fail(h, e, "upload aux");
    // fresh run: no deferred source, residual and face state restart
    const size_t cellb = h->S.qs * sizeof(double);
    cudaMemset(h->rho_last, 0, cellb);
    if (!hasH) {
        double *pf[] = {h->S.xfFx, h->S.xfFy, h->S.yfFx, h->S.yfFy};
        for (auto p : pf) cudaMemset(p, 0, cellb);
    }
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(h, e, "upload");
    h->pending = 0;
    h->gcur = 0;
    h->steps = 0;
    return DUGKS_OK;
}

extern "C" int dugks_gpu_init(dugks_handle_t *h, int kind, const double *params, int nparams, uint64_t seed) {
    dugks::TraceRange trace("dugks_gpu_init");
    if (!h) return fail(nullptr, DUGKS_EINVAL, "null handle");
    std::vector<double> f, hd, aux;
    int rc = host_init_state(h->P, h->iM, kind, params, nparams, seed, f, hd, aux);
    if (rc) return fail(h, rc, "unknown init kind or bad parameters for this model");
    rc = dugks_gpu_upload(h, f.data(), hd.empty() ? nullptr : hd.data(), aux.data());
    if (rc == DUGKS_OK) {
        h->init_kind = kind;
        h->init_radius = (nparams >= 1 && params && params[0] >= 0) ? params[0] : 0.36 * h->P.nx;
    }
    return rc;
}

extern "C" int dugks_gpu_step(dugks_handle_t *h, int nsteps, void *stream) {
    dugks::TraceRange trace("dugks_gpu_step");
    if (!h) return fail(nullptr, DUGKS_EINVAL, "null handle");
    if (nsteps < 0) return fail(h, DUGKS_EINVAL, "nsteps < 0");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (st != h->last_stream) {
        // order the new stream after the previous one
        cudaError_t e = cudaStreamSynchronize(h->last_stream);
        if (e != cudaSuccess) return cuda_fail(h, e, "stream switch");
        h->last_stream = st;
    }
    if (h->pp32) {
        for (int s = 0; s < nsteps; ++s) {
            cudaError_t e;
            if (h->pp_stream) {
                f32::PPV out = h->PPs.alt;
                out.rho = h->PPs.rho_o;
                e = f32::launch_pp32_stream(h->PPc, f32::pp_current(h->PPs), out, h->PPs.Fx, h->PPs.Fy, h->PPs.p,
                                            h->PPs.qs, h->pp_pending, st, &h->launches);
            } else {
                e = f32::launch_pp32_step(h->PPc, h->PPs, h->pp_pending, st, &h->launches, (uint32_t)(h->steps + s));
            }
            if (e != cudaSuccess) return cuda_fail(h, e, "fp32 pseudopotential step launch");
            h->pp_pending = 1;
            pp32_swap(h);  // the copy the step wrote is the state
        }
        h->steps += nsteps;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(h, e, "step launch");
        return DUGKS_OK;
    }
    if (h->fp32) {
        for (int s = 0; s < nsteps; ++s) {
            const uint32_t sn = (uint32_t)(h->steps + s);
            // FP32 storage: the streaming kernel (UW: the four-launch upwind step); the FP64
            // instance of the fused step: the tile kernel
            cudaError_t e;
            if (h->fused64)
                e = f32::launch_stepX(h->P64f, h->S64f, h->first, h->gcur, h->gcur ^ 1, st, &h->launches, sn);
            else if (h->uw32)
                e = f32::launch_uw32(h->P32, h->S32, h->uw32, h->first, st, &h->launches);
            else
                e = f32::launch_stream32(h->P32, h->S32, h->first, h->gcur, h->gcur ^ 1, st, &h->launches, sn,
                                         h->has_tmap ? &h->tmap : nullptr, h->S32.df == h->tmap_base ? 0 : f32::PL_N,
                                         h->kerr);
            if (e != cudaSuccess) return cuda_fail(h, e, "fp32 step launch");
            if (h->fused64) f32::swap_io(h->S64f);
            else f32::swap_io(h->S32);
            h->gcur ^= 1;
            h->first = 0;
        }
        h->steps += nsteps;
        if (nsteps) h->macros_fresh = false;
        return DUGKS_OK;
    }
    for (int s = 0; s < nsteps; ++s) {
        step_launcher(h)(h->P, h->S, h->pending, h->gcur, h->gcur ^ 1, st, &h->launches, nullptr);
        h->gcur ^= 1;
        h->pending = 1;
    }
    h->steps += nsteps;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(h, e, "step launch");
    return DUGKS_OK;
}

extern "C" int dugks_gpu_step_profiled(dugks_handle_t *h, int nsteps, void *stream, double *ms, int *nph) {
    if (!h || !ms || !nph) return fail(h, DUGKS_EINVAL, "null argument");
    if (h->fp32 || h->pp32) {  // phase 0 is the whole step
        int rc0 = dugks_gpu_step(h, 0, stream);
        if (rc0) return rc0;
        cudaStream_t st0 = static_cast<cudaStream_t>(stream);
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, st0);
        int rc = dugks_gpu_step(h, nsteps, stream);
        cudaEventRecord(b, st0);
        cudaError_t e = cudaEventSynchronize(b);
        float t = 0;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        if (rc) return rc;
        if (e != cudaSuccess) return cuda_fail(h, e, "profiled step");
        ms[0] = t;
        *nph = 1;
        return DUGKS_OK;
    }
    int rc = dugks_gpu_step(h, 0, stream);  // adopt the stream
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaEvent_t ev[4];
    for (auto &e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) return cuda_fail(h, cudaGetLastError(), "event create");
    double acc[3] = {0, 0, 0};
    cudaError_t e = cudaSuccess;
    for (int s = 0; s < nsteps && e == cudaSuccess; ++s) {
        step_launcher(h)(h->P, h->S, h->pending, h->gcur, h->gcur ^ 1, st, &h->launches, ev);
        h->gcur ^= 1;
        h->pending = 1;
        h->steps += 1;
        e = cudaEventSynchronize(ev[3]);
        for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
            float t = 0;
            e = cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
            acc[k] += t;
        }
    }
    for (auto &x : ev) cudaEventDestroy(x);
    if (e != cudaSuccess) return cuda_fail(h, e, "profiled step");
    for (int k = 0; k < 3; ++k) ms[k] = acc[k];
    *nph = 3;
    return DUGKS_OK;
}

static int finalize(dugks_handle *h) {
    if (!h->pending) return DUGKS_OK;
    (h->cs.precision == DUGKS_FP64_FMA ? fast::launch_fp64_finalize : exact::launch_fp64_finalize)(
        h->P, h->S, h->gcur, h->last_stream, &h->launches);
    h->pending = 0;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(h, e, "finalize launch");
    return DUGKS_OK;
}

extern "C" int dugks_gpu_reduce(dugks_handle_t *h, dugks_reductions_t *r) {
    dugks::TraceRange trace("dugks_gpu_reduce");
    if (!h || !r) return fail(h, DUGKS_EINVAL, "null argument");
    const bool hasH = (h->P.model == AC || h->P.model == HCZ);
    if (h->fp32) {
        int rc = macros_fp32(h);
        if (rc) return rc;
    }
    launch_reduce(h->P, h->S.fld[F_RHO], h->S.fld[F_PHI], h->rho_last, h->partial, h->nblocks, h->out4, hasH ? 1 : 0,
                  h->last_stream, &h->launches);
    double o[4];
    cudaError_t e = cudaMemcpyAsync(o, h->out4, sizeof o, cudaMemcpyDeviceToHost, h->last_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->last_stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "reduce");
    if (int rc = stage_loads_ok(h)) return rc;
    r->sum_rho = o[0];
    r->sum_phi = o[1];
    r->residual = std::sqrt(o[2] / (o[3] + 1.0E-30));
    r->steps = h->steps;
    return DUGKS_OK;
}

static bool is_msrc_field(const Params &P, int f) {
    if (P.model == AC || P.model == HCZ) return f >= F_PHIX && f <= F_PPV;
    return f == F_FX || f == F_FY;
}

extern "C" int dugks_gpu_get_field(dugks_handle_t *h, int field, double *out) {
    if (!h || !out || field < 0 || field >= NFIELDS) return fail(h, DUGKS_EINVAL, "bad field or null pointer");
    if (h->pp32) {
        int rc = sync_last(h);
        if (rc) return rc;
        if (field == F_RHO || field == F_U || field == F_V || field == F_P || field == F_PHI) {
            cudaError_t e = to_host(h, out, h->S.fld[field]);
            if (e != cudaSuccess) return cuda_fail(h, e, "download field");
            return DUGKS_OK;
        }
        if (field == F_FX || field == F_FY) {  // the cell force of the current psi
            cudaError_t e = f32::launch_pp32_force(h->PPc, h->PPs, h->last_stream, &h->launches);
            if (e != cudaSuccess) return cuda_fail(h, e, "force launch");
            return pp32_plane_to_host(h, field == F_FX ? h->PPs.Fx : h->PPs.Fy, out);
        }
        if (field == F_PSI) return pp32_plane_to_host(h, h->PPs.psi, out);
        if (field == F_SCG) return pp32_plane_to_host(h, h->PPs.scg, out);
        if (field == F_TAU) {
            for (size_t k = 0; k < (size_t)h->P.nx * h->P.ny; ++k) out[k] = h->P.Tau0;
            return DUGKS_OK;
        }
        return fail(h, DUGKS_EINVAL, "FP32 pseudopotential storage exposes rho, u, v, p, psi, G, tau, Fx, Fy");
    }
    if (h->fp32) {
        const bool forces = field == F_TAU || field == F_FX || field == F_FY;
        if (!(field == F_RHO || field == F_U || field == F_V || field == F_P || field == F_PHI || forces))
            return fail(h, DUGKS_EINVAL, "FP32 storage exposes rho, u, v, p, phi, tau, Fx and Fy");
        int rc = macros_fp32(h);
        if (rc) return rc;
        const double *src = h->S.fld[field];
        if (forces) {
            const size_t plane = (size_t)h->P.pitch * h->P.ny;
            if (!h->out3) {
                cudaError_t e = cudaMalloc(&h->out3, 3 * plane * sizeof(double));
                if (e != cudaSuccess) return cuda_fail(h, e, "output buffer");
            }
            double *t = h->out3, *fx = t + plane, *fy = fx + plane;
            if (h->fused64)
                f32::launch_out_forces(h->P64f, h->S64f, h->S.fld[F_PHI], h->S.fld[F_RHO], h->P.pitch, h->first, t,
                                       fx, fy, h->last_stream, &h->launches);
            else
                f32::launch_out_forces(h->P32, h->S32, h->S.fld[F_PHI], h->S.fld[F_RHO], h->P.pitch, h->first, t, fx,
                                       fy, h->last_stream, &h->launches);
            src = field == F_TAU ? t : (field == F_FX ? fx : fy);
        }
        if ((rc = sync_last(h))) return rc;
        cudaError_t e = to_host(h, out, src);
        if (e != cudaSuccess) return cuda_fail(h, e, "download field");
        return DUGKS_OK;
    }
    if (is_msrc_field(h->P, field)) {
        int rc = finalize(h);
        if (rc) return rc;
    }
    int rc = sync_last(h);
    if (rc) return rc;
    cudaError_t e = to_host(h, out, h->S.fld[field]);
    if (e != cudaSuccess) return cuda_fail(h, e, "download field");
    return DUGKS_OK;
}

extern "C" int dugks_gpu_set_field(dugks_handle_t *h, int field, const double *in) {
    if (!h || !in || field < 0 || field >= NFIELDS) return fail(h, DUGKS_EINVAL, "bad field or null pointer");
    if (h->fp32) return fail(h, DUGKS_EINVAL, "FP32 storage: set the state with dugks_gpu_upload");
    int rc = finalize(h);
    if (rc) return rc;
    if ((rc = sync_last(h))) return rc;
    cudaError_t e = to_dev(h, h->S.fld[field], in);
    if (e != cudaSuccess) return cuda_fail(h, e, "upload field");
    return DUGKS_OK;
}

extern "C" int dugks_gpu_get_dist(dugks_handle_t *h, int which, double *out) {
    if (!h || !out || which < 0 || which > 1) return fail(h, DUGKS_EINVAL, "bad argument");
    if (which == 1 && !(h->P.model == AC || h->P.model == HCZ))
        return fail(h, DUGKS_EINVAL, "model has no h distribution");
    int rc = sync_last(h);
    if (rc) return rc;
    const size_t n = (size_t)h->P.nx * h->P.ny;
    if (h->pp32) {
        // f_q = e_q rho + g_q
        std::vector<double> rho(n);
        cudaError_t e = to_host(h, rho.data(), h->PPs.rho);
        if (e != cudaSuccess) return cuda_fail(h, e, "download density");
        for (int q = 0; q < h->P.Q; ++q) {
            int rc2 = pp32_plane_to_host(h, h->PPs.df + (size_t)q * h->PPs.qs, out + q * n);
            if (rc2) return rc2;
            const double eq = h->PPc.erest[q];
            for (size_t k = 0; k < n; ++k) out[q * n + k] += eq * rho[k];
        }
        return DUGKS_OK;
    }
    if (h->fp32) {
        const size_t es = h->fused64 ? sizeof(double) : sizeof(float);
        const char *base = h->fused64 ? reinterpret_cast<const char *>(h->S64f.df)
                                      : reinterpret_cast<const char *>(h->S32.df);
        const size_t qs = h->fused64 ? h->S64f.qs : h->S32.qs;
        std::vector<unsigned char> tmp(n * es);
        // plane k of the copy the next step reads, as doubles
        auto plane = [&](int k, double *dst) -> int {
            cudaError_t e = cudaMemcpy2D(tmp.data(), (size_t)h->P.nx * es, base + (size_t)k * qs * es,
                                         (size_t)h->P.pitch * es, (size_t)h->P.nx * es, h->P.ny, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return cuda_fail(h, e, "download distribution");
            for (size_t i = 0; i < n; ++i)
                dst[i] = h->fused64 ? reinterpret_cast<const double *>(tmp.data())[i]
                                    : (double)reinterpret_cast<const float *>(tmp.data())[i];
            return DUGKS_OK;
        };
        if (which == 0) {
            for (int q = 0; q < 9; ++q) {
                int rc2 = plane(f32::PL_F + q, out + q * n);
                if (rc2) return rc2;
                const double r0 = f_rest(h->P, q);
                for (size_t k = 0; k < n; ++k) out[q * n + k] += r0;
            }
            return DUGKS_OK;
        }
        // h_q = w_q phi + g_q, h_0 = w_0 phi - sum_{q>0} g_q
        std::vector<double> phi(n), lo(n);
        int rc2 = plane(f32::PL_PHI, phi.data());
        if (!rc2) rc2 = plane(f32::PL_PHI + 1, lo.data());
        if (rc2) return rc2;
        for (size_t k = 0; k < n; ++k) phi[k] += lo[k];
        std::vector<double> gsum(n, 0.0);
        for (int q = 1; q < 9; ++q) {
            if ((rc2 = plane(f32::PL_G + q - 1, out + q * n))) return rc2;
            const double wq = h->P.omega[q];
            for (size_t k = 0; k < n; ++k) {
                gsum[k] += out[q * n + k];
                out[q * n + k] += wq * phi[k];
            }
        }
        for (size_t k = 0; k < n; ++k) out[k] = h->P.omega[0] * phi[k] - gsum[k];
        return DUGKS_OK;
    }
    for (int q = 0; q < h->P.Q; ++q) {
        cudaError_t e = to_host(h, out + q * n, (which ? h->S.h : h->S.f) + q * h->S.qs);
        if (e != cudaSuccess) return cuda_fail(h, e, "download distribution");
    }
    return DUGKS_OK;
}

// AC_Drop_L2Norm (Ark/Cpp/Output.cpp:226-238): the phase field downloaded, then the
// sums in the reference's cell order (CellArray order of a Cartesian mesh is j nx + i)
// with the drop profile of AnalyticalPhiAC_Drop (Ark/Cpp/Preprocess.cpp:402-438) at
// the cell centres (i + 1/2, j + 1/2): the same value as the reference's output.
extern "C" int dugks_gpu_drop_l2(dugks_handle_t *h, double *l2) {
    if (!h || !l2) return fail(h, DUGKS_EINVAL, "null argument");
    const Params &P = h->P;
    if (!(P.model == AC || P.model == HCZ) || !(h->init_kind == 0 || h->init_kind == 1))
        return fail(h, DUGKS_EINVAL, "the drop L2 norm needs an Allen-Cahn case initialised as a drop");
    const int nx = P.nx, ny = P.ny;
    std::vector<double> phi((size_t)nx * ny);
    int rc = dugks_gpu_get_field(h, F_PHI, phi.data());
    if (rc) return rc;
    const double centerX = 0.5 * nx, centerY = 0.5 * nx, radius = h->init_radius;
    double SumdPhi = 0.0, SumPhi_A = 0.0;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const double x = i + 0.5, y = j + 0.5;
            const double r = std::sqrt((x - centerX) * (x - centerX) + (y - centerY) * (y - centerY));
            // kind 1 (heavy phase inside) flips the profile's sign
            const double Phi_A = 0.5 * (P.PhiL + P.PhiV) +
                                 0.5 * (P.PhiL - P.PhiV) * std::tanh((h->init_kind == 1 ? radius - r : r - radius) * 2 / P.wI);
            const double dPhi = phi[(size_t)j * nx + i] - Phi_A;
            SumdPhi += dPhi * dPhi;
            SumPhi_A += Phi_A * Phi_A;
        }
    *l2 = std::sqrt(SumdPhi / SumPhi_A);
    return DUGKS_OK;
}

// thermoPressure (Ark/Cpp/Output.cpp:146-163) of every cell, from the state the last
// step's MacroSource saw (Ark/Cpp/DUGKS2DSolver.cpp:288-295): phi, p, Rho_x, Rho_y and
// the 9-point Laplacian of phi (Ark/Cpp/GradScheme.cpp:347-376) in the reference's
// operand order.  Plain FP64 handles take Rho_x, Rho_y and the wall ghost rows from
// the device's MacroSource; FP32 storage recomputes them from phi on the host (the
// gradient of Ark/Lib/GradSchemeBasic.h:153-180 with apsi = 4, bpsi = 1).  Either
// way a walled grid's ghost rows are the ones the last step extrapolated from the
// phase field it started with, as the reference's shadow cells
// (Ark/Cpp/Boundary.cpp:38-63, Ark/Cpp/DUGKS2DSolver.cpp:188).
extern "C" int dugks_gpu_thermo_pressure(dugks_handle_t *h, double *tp) {
    if (!h || !tp) return fail(h, DUGKS_EINVAL, "null argument");
    const Params &P = h->P;
    if (!(P.model == AC || P.model == HCZ)) return fail(h, DUGKS_EINVAL, "the thermodynamic pressure needs an Allen-Cahn case");
    const int nx = P.nx, ny = P.ny;
    const size_t n = (size_t)nx * ny;
    std::vector<double> phi(n), p(n), rx(n), ry(n), gb(nx), gt(nx);
    int rc = dugks_gpu_get_field(h, F_PHI, phi.data());
    if (!rc) rc = dugks_gpu_get_field(h, F_P, p.data());
    if (!rc && !h->fp32) rc = dugks_gpu_get_field(h, F_RHOX, rx.data());
    if (!rc && !h->fp32) rc = dugks_gpu_get_field(h, F_RHOY, ry.data());
    if (rc) return rc;
    if (P.walls && !h->fp32) {
        cudaError_t e = cudaMemcpy(gb.data(), h->S.gphi + (size_t)(h->gcur * 2 + 0) * P.pitch, nx * sizeof(double),
                                   cudaMemcpyDeviceToHost);
        if (e == cudaSuccess)
            e = cudaMemcpy(gt.data(), h->S.gphi + (size_t)(h->gcur * 2 + 1) * P.pitch, nx * sizeof(double),
                           cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(h, e, "ghost rows");
    } else if (P.walls) {
        // FP32 storage: the ghost rows as (head, tail) pairs
        if ((rc = sync_last(h))) return rc;
        for (int side = 0; side < 2; ++side) {
            const size_t row = f32::gphi_row(h->gcur, side);
            std::vector<double> &dst = side ? gt : gb;
            cudaError_t e = cudaSuccess;
            if (h->fused64) {
                std::vector<double> hd(2 * (size_t)nx);
                for (int k = 0; k < 2 && e == cudaSuccess; ++k)
                    e = cudaMemcpy(hd.data() + (size_t)k * nx, h->S64f.gphi + (row + k) * h->P64f.pitch,
                                   nx * sizeof(double), cudaMemcpyDeviceToHost);
                for (int i = 0; i < nx; ++i) dst[i] = hd[i] + hd[(size_t)nx + i];
            } else {
                std::vector<float> hf(2 * (size_t)nx);
                for (int k = 0; k < 2 && e == cudaSuccess; ++k)
                    e = cudaMemcpy(hf.data() + (size_t)k * nx, h->S32.gphi + (row + k) * h->P32.pitch,
                                   nx * sizeof(float), cudaMemcpyDeviceToHost);
                for (int i = 0; i < nx; ++i) dst[i] = (double)hf[i] + (double)hf[(size_t)nx + i];
            }
            if (e != cudaSuccess) return cuda_fail(h, e, "ghost rows");
        }
    }
    auto at = [&](int jj, int ii) -> double {
        ii = ii < 0 ? ii + nx : (ii >= nx ? ii - nx : ii);
        if (jj < 0) return P.walls ? gb[ii] : phi[(size_t)(ny - 1) * nx + ii];
        if (jj >= ny) return P.walls ? gt[ii] : phi[ii];
        return phi[(size_t)jj * nx + ii];
    };
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const size_t k = (size_t)j * nx + i;
            const double ph = phi[k], E = at(j, i + 1), W = at(j, i - 1), N = at(j + 1, i), S = at(j - 1, i);
            const double NE = at(j + 1, i + 1), NW = at(j + 1, i - 1), SW = at(j - 1, i - 1), SE = at(j - 1, i + 1);
            if (h->fp32) {
                double gx = (4 * (E - W) + 1 * (NE - NW + SE - SW)) / (P._2dx * 6);
                double gy = (4 * (N - S) + 1 * (NE - SE + NW - SW)) / (P._2dy * 6);
                if (std::fabs(gx) < 1.0e-14) gx = 0.0;  // SetZero (Ark/Header/Mesh_2D.h)
                if (std::fabs(gy) < 1.0e-14) gy = 0.0;
                rx[k] = P.aPhi * gx;
                ry[k] = P.aPhi * gy;
            }
            const double lap = (4 * (E + N + W + S) + (NE + NW + SW + SE) - 20 * ph) / (6 * P.MinL * P.MinL);
            const double sq = (rx[k] * rx[k] + ry[k] * ry[k]) / (P.aPhi * P.aPhi);
            const double pZero = ph * 2 * P.Beta * (ph - P.PhiL) * (ph - P.PhiV) * (2 * ph - P.PhiL - P.PhiV) -
                                 P.Beta * (ph - P.PhiL) * (ph - P.PhiL) * (ph - P.PhiV) * (ph - P.PhiV);
            tp[k] = pZero - P.Kappa * ph * lap + P.Kappa * sq / 2 + p[k];
        }
    return DUGKS_OK;
}

extern "C" int dugks_gpu_download(dugks_handle_t *h, double *rho, double *u, double *v, double *phi, double *p) {
    dugks::TraceRange trace("dugks_gpu_download");
    if (!h) return fail(nullptr, DUGKS_EINVAL, "null handle");
    double *dst[5] = {rho, u, v, phi, p};
    const int fid[5] = {F_RHO, F_U, F_V, F_PHI, F_P};
    for (int k = 0; k < 5; ++k)
        if (dst[k]) {
            int rc = dugks_gpu_get_field(h, fid[k], dst[k]);
            if (rc) return rc;
        }
    return DUGKS_OK;
}

extern "C" int dugks_gpu_check_finite(dugks_handle_t *h) {
    if (!h) return fail(nullptr, DUGKS_EINVAL, "null handle");
    const Params &P = h->P;
    cudaStream_t st = h->last_stream;
    cudaMemsetAsync(h->flag, 0, sizeof(int), st);
    const bool hasH = (P.model == AC || P.model == HCZ);
    if (h->pp32) {
        const size_t qs = (size_t)P.pitch * P.ny;
        const int fids[4] = {F_RHO, F_U, F_V, F_P};
        for (int k : fids) launch_check_finite(h->S.fld[k], qs, h->flag, st, &h->launches);
    } else if (h->fp32) {
        int rc = macros_fp32(h);
        if (rc) return rc;
        const size_t qs = (size_t)P.pitch * P.ny;
        const int fids[5] = {F_RHO, F_U, F_V, F_P, F_PHI};
        for (int k : fids) launch_check_finite(h->S.fld[k], qs, h->flag, st, &h->launches);
    } else {
        launch_check_finite(h->S.f, (size_t)P.Q * h->S.qs, h->flag, st, &h->launches);
        if (hasH) launch_check_finite(h->S.h, (size_t)P.Q * h->S.qs, h->flag, st, &h->launches);
        launch_check_finite(h->S.fld[F_RHO], h->S.qs, h->flag, st, &h->launches);
    }
    int flag = 0;
    cudaError_t e = cudaMemcpyAsync(&flag, h->flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(h, e, "check_finite");
    if (int rc = stage_loads_ok(h)) return rc;
    return flag ? fail(h, DUGKS_ENAN, "non-finite value in the state") : DUGKS_OK;
}

extern "C" int dugks_gpu_last_error(const dugks_handle_t *h, char *buf, size_t len) {
    if (!buf || len == 0) return DUGKS_EINVAL;
    const std::string &s = h ? h->err : g_create_err;
    std::snprintf(buf, len, "%s", s.c_str());
    return DUGKS_OK;
}

extern "C" int64_t dugks_gpu_launch_count(const dugks_handle_t *h) { return h ? h->launches : 0; }

// ---- checkpoint / restart
namespace {
struct CkptHeader {
    char magic[8];
    uint32_t version, header_bytes;
    dugks_case_t cs;
    dugks_grid_t grid;
    int32_t pad0;
    uint64_t arena_bytes;
    int64_t steps;
    int32_t pending, gcur, first, pp_pending, orient, pad1;
    f32::PPP ppc;
};
const char CKPT_MAGIC[8] = {'D', 'U', 'G', 'K', 'S', 'C', 'K', '3'};

// orientation of the fused path's ping-pong views: 0 as created, 1 swapped
int fused_orient(const dugks_handle *h) {
    if (h->pp32) return h->PPs.rho == h->pp_rho0 ? 0 : 1;
    if (!h->fp32) return 0;
    const void *df = h->fused64 ? static_cast<const void *>(h->S64f.df) : static_cast<const void *>(h->S32.df);
    return df == static_cast<const void *>(h->arena) ? 0 : 1;
}
}  // namespace

extern "C" int dugks_gpu_checkpoint_bytes(const dugks_handle_t *h, size_t *bytes) {
    if (!h || !bytes) return DUGKS_EINVAL;
    *bytes = sizeof(CkptHeader) + h->arena_bytes;
    return DUGKS_OK;
}

extern "C" int dugks_gpu_step_count(const dugks_handle_t *h, int64_t *steps) {
    if (!h || !steps) return DUGKS_EINVAL;
    *steps = h->steps;
    return DUGKS_OK;
}

extern "C" int dugks_gpu_checkpoint(dugks_handle_t *h, void *buf, size_t len) {
    dugks::TraceRange trace("dugks_gpu_checkpoint");
    if (!h || !buf) return fail(h, DUGKS_EINVAL, "null argument");
    if (len < sizeof(CkptHeader) + h->arena_bytes) return fail(h, DUGKS_EINVAL, "checkpoint buffer too small");
    int rc = sync_last(h);
    if (rc) return rc;
    CkptHeader hd{};
    std::memcpy(hd.magic, CKPT_MAGIC, sizeof hd.magic);
    hd.version = 1;
    hd.header_bytes = sizeof(CkptHeader);
    hd.cs = h->cs;
    hd.grid = h->grid;
    hd.arena_bytes = h->arena_bytes;
    hd.steps = h->steps;
    hd.pending = h->pending;
    hd.gcur = h->gcur;
    hd.first = h->first;
    hd.pp_pending = h->pp_pending;
    hd.orient = fused_orient(h);
    hd.ppc = h->PPc;
    std::memcpy(buf, &hd, sizeof hd);
    cudaError_t e = cudaMemcpy(static_cast<char *>(buf) + sizeof hd, h->arena, h->arena_bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(h, e, "checkpoint copy");
    return DUGKS_OK;
}

extern "C" int dugks_gpu_restore(dugks_handle_t *h, const void *buf, size_t len) {
    dugks::TraceRange trace("dugks_gpu_restore");
    if (!h || !buf) return fail(h, DUGKS_EINVAL, "null argument");
    CkptHeader hd;
    if (len < sizeof hd) return fail(h, DUGKS_EINVAL, "checkpoint buffer too small");
    std::memcpy(&hd, buf, sizeof hd);
    if (std::memcmp(hd.magic, CKPT_MAGIC, sizeof hd.magic) != 0 || hd.version != 1 ||
        hd.header_bytes != sizeof(CkptHeader))
        return fail(h, DUGKS_EINVAL, "not a checkpoint of this library version");
    if (std::memcmp(&hd.cs, &h->cs, sizeof hd.cs) != 0 || std::memcmp(&hd.grid, &h->grid, sizeof hd.grid) != 0 ||
        hd.arena_bytes != h->arena_bytes)
        return fail(h, DUGKS_EINVAL, "checkpoint of a different case or grid");
    if (len < sizeof hd + hd.arena_bytes) return fail(h, DUGKS_EINVAL, "truncated checkpoint");
    int rc = sync_last(h);
    if (rc) return rc;
    cudaError_t e =
        cudaMemcpy(h->arena, static_cast<const char *>(buf) + sizeof hd, h->arena_bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(h, e, "restore copy");
    h->steps = hd.steps;
    h->pending = hd.pending;
    h->gcur = hd.gcur;
    h->first = hd.first;
    h->pp_pending = hd.pp_pending;
    if (h->pp32) h->PPc = hd.ppc;
    if (fused_orient(h) != hd.orient) {
        if (h->pp32) {
            pp32_swap(h);
        } else if (h->fused64) {
            f32::swap_io(h->S64f);
        } else {
            f32::swap_io(h->S32);
        }
    }
    h->macros_fresh = false;
    return DUGKS_OK;
}

extern "C" int dugks_gpu_destroy(dugks_handle_t *h) {
    if (!h) return DUGKS_OK;
    cudaStreamSynchronize(h->last_stream);
    cudaFree(h->arena);
    if (h->out3) cudaFree(h->out3);
    delete h;
    return DUGKS_OK;
}

// ---- internal interface for the serving layer (serving.cu)
namespace dugks {
namespace internal {

size_t footprint(const dugks_case_t &c, const dugks_grid_t &g) {
    Params P;
    derive_params(c, g, P);
    if (c.precision == DUGKS_FP32_DEV && (P.model == PP9 || P.model == PP16)) return pp32_arena_bytes(P);
    if (c.precision == DUGKS_FP32_DEV) return fused_arena_bytes(P, sizeof(float));
    if (c.precision == DUGKS_FP64_FUSED) return fused_arena_bytes(P, sizeof(double));
    return fp64_arena_bytes(P);
}

bool batchable(const dugks_handle_t *h) {
    return h && h->fp32 && !h->fused64 && !h->P.uw && (h->P.model == AC || h->P.model == HCZ);
}

void fp32_views(const dugks_handle_t *h, f32::P32 *P, f32::S32 *S) {
    *P = h->P32;
    *S = h->S32;
}

int64_t steps_done(const dugks_handle_t *h) { return h->steps; }
int model_of(const dugks_handle_t *h) { return h->P.model; }
int walls_of(const dugks_handle_t *h) { return h->P.walls ? 1 : 0; }
double dt_of(const dugks_handle_t *h) { return h->P.dt; }

// n steps were run outside the handle (by the batched kernel) from its current
// state with step numbers steps .. steps+n-1: adopt the ping-pong orientation,
// ghost-row buffer, first-step flag and counters those steps leave
void fp32_adopt_steps(dugks_handle_t *h, int64_t n) {
    if (n <= 0) return;
    if (n & 1) f32::swap_io(h->S32);
    h->steps += n;
    h->gcur = (int)(h->steps & 1);
    h->first = 0;
    h->macros_fresh = false;
}

void set_stream(dugks_handle_t *h, cudaStream_t st) { h->last_stream = st; }

// for the slab decomposition (slabs.cu)
void derive_fp32(const Params &P, f32::P32 *Q) { derive_p32<float>(P, *Q); }
double rest_f(const Params &P, int q) { return f_rest(P, q); }

}  // namespace internal
}  // namespace dugks
