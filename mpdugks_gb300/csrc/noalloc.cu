// dugks_gpu_step_noalloc: the FP64 Allen-Cahn step on a caller-owned device
// state, with every scratch array (f-bar-plus, x- and y-face fluxes, ghost-phi
// rows) in one fixed file-scope device array instead of memory allocated for
// the call.
//
// Who needs it: code that may not allocate device memory on its own -- a
// host application that hands this library a fixed memory budget up front
// (or owns a custom pool and forbids other allocators), a kernel-launching
// plugin inside another runtime, or a loop that must not allocate once it is
// running (allocation is a device-wide synchronising call that can also fail
// with out-of-memory mid-run).  Such callers pass their own input and output
// buffers and get the step without a cudaMalloc/cudaFree anywhere.
//
// Limits: D2Q9 Allen-Cahn models (AC, HCZ); at most NOALLOC_MAX_CELLS cells.
// The scratch array is ~2 MB and stays allocated on every GPU that loads
// the library until the process exits.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/dugks_gpu.h"
#include "dugks_device.cuh"

namespace dugks {
void derive_params(const dugks_case_t &cs, const dugks_grid_t &g, Params &P);
void set_global_error(const std::string &msg);
namespace exact {
void launch_fp64_step(const Params &P, const State &S, int do_msrc, int gin, int gout, cudaStream_t st,
                      int64_t *launches, cudaEvent_t *ev);
void launch_fp64_finalize(const Params &P, const State &S, int gin, cudaStream_t st, int64_t *launches);
}  // namespace exact
namespace fast {
void launch_fp64_step(const Params &P, const State &S, int do_msrc, int gin, int gout, cudaStream_t st,
                      int64_t *launches, cudaEvent_t *ev);
void launch_fp64_finalize(const Params &P, const State &S, int gin, cudaStream_t st, int64_t *launches);
}  // namespace fast
}  // namespace dugks

using namespace dugks;

namespace {

constexpr int NOALLOC_MAX_CELLS = 4096;  // e.g. 64 x 64
constexpr int NOALLOC_MAX_NX = 2048;
constexpr int NQ = 9;
// f-bar-plus (2Q planes), x-face fluxes (2Q planes), y-face fluxes (2Q planes of
// ny+1 rows) and four ghost-phi rows, for the largest admitted grid.
constexpr size_t NOALLOC_SCRATCH_DOUBLES =
    (size_t)NQ * (4 * NOALLOC_MAX_CELLS + 2 * (NOALLOC_MAX_CELLS + NOALLOC_MAX_NX)) + 4 * NOALLOC_MAX_NX;

// The scratch.  In host code this name is only a stand-in for the device
// symbol; its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

constexpr int MAX_DEVICES = 64;
std::mutex g_addr_mutex;
double *g_addr[MAX_DEVICES] = {};

// Device address of the scratch on the current device.  Looked up on every call
// made outside a stream capture (so a re-created context, e.g. after
// cudaDeviceReset, never sees a stale address); a call whose stream is being
// captured uses the address the last uncaptured call on this device found, and
// looks it up only if there is none yet.
cudaError_t scratch_address(cudaStream_t st, double **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(g_addr_mutex);
    if (cap == cudaStreamCaptureStatusNone || !g_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = static_cast<double *>(p);
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int dugks_gpu_step_noalloc(const dugks_case_t *c, const dugks_grid_t *g, double *d_f, double *d_h,
                                      double *d_aux, int nsteps, void *stream) {
    if (!c || !g || !d_f || !d_h || !d_aux) {
        set_global_error("dugks_gpu_step_noalloc: null argument");
        return DUGKS_EINVAL;
    }
    if (c->model != DUGKS_MODEL_AC && c->model != DUGKS_MODEL_HCZ) {
        set_global_error("dugks_gpu_step_noalloc: only the D2Q9 Allen-Cahn models (AC, HCZ) are supported");
        return DUGKS_EINVAL;
    }
    if (c->precision != DUGKS_FP64 && c->precision != DUGKS_FP64_FMA) {
        set_global_error("dugks_gpu_step_noalloc: precision must be DUGKS_FP64 or DUGKS_FP64_FMA");
        return DUGKS_EINVAL;
    }
    if (c->flux_scheme != DUGKS_FLUX_CD || (c->wall_scheme != DUGKS_WALL_BB && g->y_walls)) {
        set_global_error("dugks_gpu_step_noalloc: the CD flux scheme and bounce-back walls only (UW and NEE "
                         "need scratch)");
        return DUGKS_EINVAL;
    }
    if (g->nx < 3 || g->ny < 3 || nsteps < 0) {
        set_global_error("dugks_gpu_step_noalloc: nx, ny must be >= 3 and nsteps >= 0");
        return DUGKS_EINVAL;
    }
    const long long cells = (long long)g->nx * g->ny;
    if (cells > NOALLOC_MAX_CELLS || g->nx > NOALLOC_MAX_NX) {
        set_global_error("dugks_gpu_step_noalloc: grid of " + std::to_string(cells) +
                         " cells exceeds the fixed scratch capacity of " + std::to_string(NOALLOC_MAX_CELLS) +
                         " cells (nx <= " + std::to_string(NOALLOC_MAX_NX) + ")");
        return DUGKS_EINVAL;
    }
    if (nsteps == 0) return DUGKS_OK;
    double *base = nullptr;
    cudaError_t e = scratch_address(static_cast<cudaStream_t>(stream), &base);
    if (e != cudaSuccess) {
        set_global_error(std::string("dugks_gpu_step_noalloc: cudaGetSymbolAddress failed: ") +
                         cudaGetErrorString(e));
        return DUGKS_ECUDA;
    }
    Params P;
    derive_params(*c, *g, P);
    P.pitch = g->nx;  // caller buffers are dense [..][ny][nx]
    const size_t C = (size_t)cells, Cy = (size_t)(g->ny + 1) * g->nx;
    State S{};
    S.qs = C;
    S.qsy = Cy;
    S.f = d_f;
    S.h = d_h;
    for (int k = 0; k < NFIELDS; ++k) S.fld[k] = d_aux + (size_t)k * C;
    // every scratch element is written before it is read within one call, so
    // nothing is cleared
    double *cur = base;
    S.bf = cur; cur += NQ * C;
    S.bh = cur; cur += NQ * C;
    S.xff = cur; cur += NQ * C;
    S.xfh = cur; cur += NQ * C;
    S.yff = cur; cur += NQ * Cy;
    S.yfh = cur; cur += NQ * Cy;
    S.gphi = cur;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool fma = c->precision == DUGKS_FP64_FMA;
    int64_t launches = 0;
    int gcur = 0, pending = 0;
    for (int s = 0; s < nsteps; ++s) {
        (fma ? fast::launch_fp64_step : exact::launch_fp64_step)(P, S, pending, gcur, gcur ^ 1, st, &launches,
                                                                 nullptr);
        gcur ^= 1;
        pending = 1;
    }
    // leave a complete state: the last step's MacroSource is applied here
    (fma ? fast::launch_fp64_finalize : exact::launch_fp64_finalize)(P, S, gcur, st, &launches);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_global_error(std::string("dugks_gpu_step_noalloc: launch failed: ") + cudaGetErrorString(e));
        return DUGKS_ECUDA;
    }
    return DUGKS_OK;
}
