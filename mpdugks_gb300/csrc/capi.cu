// C ABI of libdugks_gpu.so (declared in include/dugks_gpu.h).
//
// Host side of the drop-in: derives the case constants with the reference's
// header formulas, allocates the resident device state, runs the reference's
// initialisation functions on the host, and drives the step kernels.
#include <cuda_runtime.h>

#include <cmath>
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
    void set_d2v16_matrix(const double *m256, cudaStream_t st);                                                 \
    void launch_fp64_step(const Params &P, const State &S, int do_msrc, int gin, int gout, cudaStream_t st,     \
                          int64_t *launches, cudaEvent_t *ev);                                                  \
    void launch_fp64_finalize(const Params &P, const State &S, int gin, cudaStream_t st, int64_t *launches);   \
    void launch_reduce(const Params &P, const double *rho, const double *phi, double *rho_last, double *partial, \
                       int nblocks, double *out4, int has_phi, cudaStream_t st, int64_t *launches);             \
    void launch_check_finite(const double *a, size_t n, int *flag, cudaStream_t st, int64_t *launches);         \
    }
DUGKS_DECLARE_FP64(exact)
DUGKS_DECLARE_FP64(fast)
using exact::launch_reduce;
using exact::launch_check_finite;
void build_d2v16_matrix(double c, double out[16][16]);
void derive_params(const dugks_case_t &cs, const dugks_grid_t &g, Params &P);
int host_init_state(const Params &P, const double iM[16][16], int kind, const double *params, int nparams,
                    uint64_t seed, std::vector<double> &f, std::vector<double> &h, std::vector<double> &aux);
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

extern "C" int dugks_gpu_create(const dugks_case_t *c, const dugks_grid_t *g, dugks_handle_t **out) {
    if (!c || !g || !out) return fail(nullptr, DUGKS_EINVAL, "null argument");
    *out = nullptr;
    if (g->nx < 3 || g->ny < 3) return fail(nullptr, DUGKS_EINVAL, "nx and ny must be >= 3");
    if ((long long)g->nx * g->ny > (1LL << 31)) return fail(nullptr, DUGKS_EINVAL, "grid too large");
    if (c->model < DUGKS_MODEL_AC || c->model > DUGKS_MODEL_PP16)
        return fail(nullptr, DUGKS_EINVAL, "unknown model");
    if ((c->model == DUGKS_MODEL_PP9 || c->model == DUGKS_MODEL_PP16) && g->y_walls)
        return fail(nullptr, DUGKS_EINVAL, "pseudopotential models are periodic only (faceFaces need no walls)");
    if (c->precision != DUGKS_FP64 && c->precision != DUGKS_FP32_DEV && c->precision != DUGKS_FP64_FMA)
        return fail(nullptr, DUGKS_EINVAL, "unknown precision");
    if (c->precision == DUGKS_FP32_DEV)
        return fail(nullptr, DUGKS_EINVAL, "FP32 deviation storage is served by dugks_f32_* entry points");
    dugks_handle *h = new (std::nothrow) dugks_handle();
    if (!h) return fail(nullptr, DUGKS_ENOMEM, "host allocation failed");
    h->cs = *c;
    h->grid = *g;
    derive_params(*c, *g, h->P);
    Params &P = h->P;
    if (P.model == PP16) build_d2v16_matrix(P.c16, h->iM);
    // ---- carve the arena
    const size_t rowb = (size_t)P.pitch * sizeof(double);
    const size_t cellb = align256(rowb * P.ny), ycellb = align256(rowb * (P.ny + 1));
    const int Q = P.Q;
    const bool hasH = (P.model == AC || P.model == HCZ);
    const bool pp = !hasH;
    size_t total = 0;
    total += 2 * Q * cellb;                       // f, h (h unused by PP but kept simple)
    total += 2 * Q * cellb;                       // bf, bh
    total += 2 * Q * cellb + 2 * Q * ycellb;      // x/y face fluxes
    total += NFIELDS * cellb;                     // macro fields
    total += align256(4 * rowb);                  // ghost phi rows
    if (pp) total += 14 * cellb + 2 * Q * cellb;  // pseudopotential face state + face BhDt
    total += cellb;                               // rho_last
    h->nblocks = 152 * 4;
    total += align256(sizeof(double) * 4 * h->nblocks) + 256 + 256;
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
    h->rho_last = take(cellb);
    h->partial = take(align256(sizeof(double) * 4 * h->nblocks));
    h->out4 = take(256);
    h->flag = reinterpret_cast<int *>(take(256));
    if (P.model == PP16) {
        exact::set_d2v16_matrix(&h->iM[0][0], nullptr);
        fast::set_d2v16_matrix(&h->iM[0][0], nullptr);
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
static cudaError_t to_dev(const dugks_handle *h, double *d, const double *src, int rows = -1) {
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
    if (!h) return fail(nullptr, DUGKS_EINVAL, "null handle");
    std::vector<double> f, hd, aux;
    int rc = host_init_state(h->P, h->iM, kind, params, nparams, seed, f, hd, aux);
    if (rc) return fail(h, rc, "unknown init kind or bad parameters for this model");
    rc = dugks_gpu_upload(h, f.data(), hd.empty() ? nullptr : hd.data(), aux.data());
    return rc;
}

extern "C" int dugks_gpu_step(dugks_handle_t *h, int nsteps, void *stream) {
    if (!h) return fail(nullptr, DUGKS_EINVAL, "null handle");
    if (nsteps < 0) return fail(h, DUGKS_EINVAL, "nsteps < 0");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (st != h->last_stream) {
        // order the new stream after the previous one
        cudaError_t e = cudaStreamSynchronize(h->last_stream);
        if (e != cudaSuccess) return cuda_fail(h, e, "stream switch");
        h->last_stream = st;
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
    if (!h || !r) return fail(h, DUGKS_EINVAL, "null argument");
    const bool hasH = (h->P.model == AC || h->P.model == HCZ);
    launch_reduce(h->P, h->S.fld[F_RHO], h->S.fld[F_PHI], h->rho_last, h->partial, h->nblocks, h->out4, hasH ? 1 : 0,
                  h->last_stream, &h->launches);
    double o[4];
    cudaError_t e = cudaMemcpyAsync(o, h->out4, sizeof o, cudaMemcpyDeviceToHost, h->last_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->last_stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "reduce");
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
    for (int q = 0; q < h->P.Q; ++q) {
        cudaError_t e = to_host(h, out + q * n, (which ? h->S.h : h->S.f) + q * h->S.qs);
        if (e != cudaSuccess) return cuda_fail(h, e, "download distribution");
    }
    return DUGKS_OK;
}

extern "C" int dugks_gpu_download(dugks_handle_t *h, double *rho, double *u, double *v, double *phi, double *p) {
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
    launch_check_finite(h->S.f, (size_t)P.Q * h->S.qs, h->flag, st, &h->launches);
    if (hasH) launch_check_finite(h->S.h, (size_t)P.Q * h->S.qs, h->flag, st, &h->launches);
    launch_check_finite(h->S.fld[F_RHO], h->S.qs, h->flag, st, &h->launches);
    int flag = 0;
    cudaError_t e = cudaMemcpyAsync(&flag, h->flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(h, e, "check_finite");
    return flag ? fail(h, DUGKS_ENAN, "non-finite value in the state") : DUGKS_OK;
}

extern "C" int dugks_gpu_last_error(const dugks_handle_t *h, char *buf, size_t len) {
    if (!buf || len == 0) return DUGKS_EINVAL;
    const std::string &s = h ? h->err : g_create_err;
    std::snprintf(buf, len, "%s", s.c_str());
    return DUGKS_OK;
}

extern "C" int64_t dugks_gpu_launch_count(const dugks_handle_t *h) { return h ? h->launches : 0; }

extern "C" int dugks_gpu_destroy(dugks_handle_t *h) {
    if (!h) return DUGKS_OK;
    cudaStreamSynchronize(h->last_stream);
    cudaFree(h->arena);
    delete h;
    return DUGKS_OK;
}
