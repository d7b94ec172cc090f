// Slab decomposition of one FP32-storage case along y: the data path that
// spreads a case over several GPUs (or partitions of one GPU).
//
// Partition p owns rows [row0_p, row0_p + nrows_p) of the grid and keeps two
// halo rows of device memory on each side.  A side is either a wall (the
// grid's own bounce-back wall: the first/last partition of a walled grid) or
// a halo filled from the neighbouring partition (periodic grids wrap from
// the last partition to the first).  Every step each partition runs the
// streaming kernel on its rows (halo rows are read, never written), then the
// two boundary rows of all PL_N state planes (9 f deviations, 8 phase-field
// remainders g, the phi pair, 6 aux) are copied into the neighbours' halo rows: one
// strided copy per neighbour and side.  Every cell computes from the same inputs in
// the same order as in the undivided case, so the decomposed run is bit-identical to
// the undivided one.
//
// The reference has no counterpart (one OpenMP process per case).  Only one
// GPU is exercised here: partitions on different devices use peer copies
// through the same calls, with a device synchronisation per step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dugks_gpu.h"
#include "dugks_device.cuh"
#include "fp32_state.cuh"
#include "trace.hpp"

namespace dugks {
void derive_params(const dugks_case_t &cs, const dugks_grid_t &g, Params &P);
void set_global_error(const std::string &msg);
int host_init_state(const Params &P, const double iM[16][16], int kind, const double *params, int nparams,
                    uint64_t seed, std::vector<double> &f, std::vector<double> &h, std::vector<double> &aux);
namespace internal {
void derive_fp32(const Params &P, f32::P32 *Q);
double rest_f(const Params &P, int q);
}  // namespace internal
namespace f32 {
cudaError_t launch_stream32(const P32 &P, const S32 &S, int first, int gin, int gout, cudaStream_t st,
                            int64_t *launches, uint32_t step, const void *tmap, int zin, int *err);
void launch_macros32(const P32 &P, const S32 &S, double *rho, double *u, double *v, double *p, double *phi,
                     int opitch, cudaStream_t st, int64_t *launches);
template <typename R>
cudaError_t launch_plane_from_f64(R *dst, int dpitch, const double *src, int nx, int ny, double sub,
                                  cudaStream_t st, int64_t *launches);
}  // namespace f32
namespace exact {
void launch_reduce(const Params &P, const double *rho, const double *phi, double *rho_last, double *partial,
                   int nblocks, double *out4, int has_phi, cudaStream_t st, int64_t *launches);
}  // namespace exact
}  // namespace dugks

using namespace dugks;

namespace {

constexpr int H = f32::SLAB_HALO;
constexpr int MIN_ROWS = 8;  // rows of a partition (the streaming kernel's window)
constexpr int RED_BLOCKS = 152;  // blocks of a partition's reduction

struct Part {
    int device = 0, row0 = 0, nrows = 0, lo = -1, hi = -1;  // lo/hi: neighbour partition, -1 = wall
    f32::P32 P{};
    f32::S32 S{};          // current orientation (ping-pong swapped after each step)
    float *arena = nullptr;
    double *fields = nullptr;  // rho u v p phi [5][nrows][pitch] (download)
    double *red = nullptr;     // reductions: rho_last [nrows][pitch], partial sums [RED_BLOCKS][4], totals [4]
    size_t plane = 0;          // floats per plane (nrows + 2H rows)
    cudaStream_t st = nullptr;
    bool own_stream = false;
};

bool plan(int ny, int walls, int nparts, std::vector<int> &row0, std::vector<int> &nrows, std::vector<int> &lo,
          std::vector<int> &hi) {
    if (nparts < 1 || ny < nparts * MIN_ROWS) return false;
    row0.resize(nparts);
    nrows.resize(nparts);
    lo.resize(nparts);
    hi.resize(nparts);
    for (int p = 0; p < nparts; ++p) {
        row0[p] = (int)((long long)ny * p / nparts);
        nrows[p] = (int)((long long)ny * (p + 1) / nparts) - row0[p];
        lo[p] = p > 0 ? p - 1 : (walls ? -1 : nparts - 1);
        hi[p] = p < nparts - 1 ? p + 1 : (walls ? -1 : 0);
    }
    return true;
}

// The halo copies after every step, in issue order: for each partition, its top H
// rows into the upper neighbour's lower halo, then its bottom H rows into the lower
// neighbour's upper halo.  Rows are local (0 = the first owned row).
std::vector<dugks_halo_copy_t> schedule(const std::vector<int> &nrows, const std::vector<int> &lo,
                                        const std::vector<int> &hi) {
    std::vector<dugks_halo_copy_t> out;
    for (size_t p = 0; p < nrows.size(); ++p) {
        if (hi[p] >= 0) out.push_back({(int)p, nrows[p] - H, hi[p], -H, H});
        if (lo[p] >= 0) out.push_back({(int)p, 0, lo[p], nrows[lo[p]], H});
    }
    return out;
}

}  // namespace

struct dugks_slabs {
    dugks_case_t cs{};
    dugks_grid_t grid{};
    Params P{};
    std::vector<Part> parts;
    std::vector<dugks_halo_copy_t> copies;  // the exchange schedule
    int first = 1, gcur = 0;
    int64_t steps = 0, launches = 0;
    bool multi_device = false;
};

namespace {

int fail(const std::string &m, int code = DUGKS_EINVAL) {
    set_global_error("dugks_slabs: " + m);
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    return fail(std::string(what) + ": " + cudaGetErrorString(e), DUGKS_ECUDA);
}

// rows [0, n) of the PL_N planes of `src` (stride sp floats) -> rows of `dst` (stride dp)
cudaError_t copy_rows(float *dst, size_t dp, const float *src, size_t sp, int pitch, int n, cudaStream_t st) {
    return cudaMemcpy2DAsync(dst, dp * sizeof(float), src, sp * sizeof(float), (size_t)n * pitch * sizeof(float),
                             f32::PL_N, cudaMemcpyDefault, st);
}

// halo exchange into the current state of every partition, as the schedule lists it
cudaError_t exchange(dugks_slabs *s) {
    const int pitch = s->P.pitch;
    for (const auto &c : s->copies) {
        const Part &p = s->parts[c.src];
        Part &q = s->parts[c.dst];
        cudaSetDevice(q.device);
        cudaError_t e = copy_rows(q.S.df + (ptrdiff_t)c.dst_row * pitch, q.plane, p.S.df + (ptrdiff_t)c.src_row * pitch,
                                  p.plane, pitch, c.rows, q.st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t sync_all(dugks_slabs *s) {
    for (auto &p : s->parts) {
        cudaSetDevice(p.device);
        cudaError_t e = cudaStreamSynchronize(p.st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace

extern "C" int dugks_slabs_plan(int ny, int y_walls, int nparts, int *row0, int *nrows, int *lo, int *hi) {
    std::vector<int> a, b, c, d;
    if (!row0 || !nrows || !lo || !hi) return fail("null argument");
    if (!plan(ny, y_walls, nparts, a, b, c, d))
        return fail("cannot split " + std::to_string(ny) + " rows into " + std::to_string(nparts) +
                    " partitions of at least " + std::to_string(MIN_ROWS) + " rows");
    for (int p = 0; p < nparts; ++p) {
        row0[p] = a[p];
        nrows[p] = b[p];
        lo[p] = c[p];
        hi[p] = d[p];
    }
    return DUGKS_OK;
}

extern "C" int dugks_slabs_schedule(int ny, int y_walls, int nparts, dugks_halo_copy_t *out, int max, int *count) {
    std::vector<int> row0, nrows, lo, hi;
    if (!count || !plan(ny, y_walls, nparts, row0, nrows, lo, hi))
        return fail("schedule: needs count and at least " + std::to_string(MIN_ROWS) + " rows per partition");
    const std::vector<dugks_halo_copy_t> c = schedule(nrows, lo, hi);
    *count = (int)c.size();
    if (out) {
        if (max < (int)c.size()) return fail("schedule: output holds fewer copies than the schedule");
        std::copy(c.begin(), c.end(), out);
    }
    return DUGKS_OK;
}

extern "C" int dugks_slabs_create(const dugks_case_t *c, const dugks_grid_t *g, int nparts, const int *devices,
                                  dugks_slabs_t **out) {
    if (!c || !g || !out) return fail("null argument");
    *out = nullptr;
    if (c->precision != DUGKS_FP32_DEV || !(c->model == DUGKS_MODEL_AC || c->model == DUGKS_MODEL_HCZ) ||
        c->flux_scheme != DUGKS_FLUX_CD || (c->wall_scheme != DUGKS_WALL_BB && g->y_walls))
        return fail("slab decomposition runs FP32-storage Allen-Cahn cases (AC, HCZ) with the CD flux scheme "
                    "and bounce-back walls");
    if (g->nx < 3) return fail("nx must be >= 3");
    std::vector<int> row0, nrows, lo, hi;
    if (!plan(g->ny, g->y_walls, nparts, row0, nrows, lo, hi))
        return fail("cannot split " + std::to_string(g->ny) + " rows into " + std::to_string(nparts) +
                    " partitions of at least " + std::to_string(MIN_ROWS) + " rows");
    auto *s = new dugks_slabs();
    s->cs = *c;
    s->grid = *g;
    derive_params(*c, *g, s->P);
    s->parts.resize(nparts);
    s->copies = schedule(nrows, lo, hi);
    int dev0 = 0;
    cudaGetDevice(&dev0);
    for (int p = 0; p < nparts; ++p) {
        Part &q = s->parts[p];
        q.device = devices ? devices[p] : dev0;
        if (q.device != s->parts[0].device) s->multi_device = true;
        q.row0 = row0[p];
        q.nrows = nrows[p];
        q.lo = lo[p];
        q.hi = hi[p];
        internal::derive_fp32(s->P, &q.P);
        q.P.ny = q.nrows;
        q.P.walls = 1;  // the wall / halo instance; halo flags pick the sides
        q.P.row0 = q.row0;
        q.P.halo_lo = q.lo >= 0;
        q.P.halo_hi = q.hi >= 0;
        const int pitch = s->P.pitch;
        q.plane = (size_t)(q.nrows + 2 * H) * pitch;
        // two state sets of PL_N planes, 12 first-step planes, ghost phi rows
        const size_t floats = 2 * f32::PL_N * q.plane + f32::I_N * q.plane + f32::GPHI_ROWS * (size_t)pitch;
        cudaError_t e = cudaSetDevice(q.device);
        // one stream per device: the partitions of a device, their halo copies and
        // the next step are ordered on it
        for (int r = 0; r < p && e == cudaSuccess; ++r)
            if (s->parts[r].device == q.device) q.st = s->parts[r].st;
        if (e == cudaSuccess && !q.st) {
            e = cudaStreamCreateWithFlags(&q.st, cudaStreamNonBlocking);
            if (e == cudaSuccess) q.own_stream = true;
        }
        if (e == cudaSuccess) e = cudaMalloc(&q.arena, floats * sizeof(float));
        if (e == cudaSuccess) e = cudaMalloc(&q.fields, 5 * (size_t)q.nrows * pitch * sizeof(double));
        const size_t red = (size_t)q.nrows * pitch + 4 * RED_BLOCKS + 4;
        if (e == cudaSuccess) e = cudaMalloc(&q.red, red * sizeof(double));
        if (e == cudaSuccess) e = cudaMemsetAsync(q.red, 0, red * sizeof(double), q.st);
        if (e == cudaSuccess) e = cudaMemsetAsync(q.arena, 0, floats * sizeof(float), q.st);
        if (e != cudaSuccess) {
            dugks_slabs_destroy(s);
            return cuda_fail(e, "partition allocation");
        }
        float *a = q.arena + (size_t)H * pitch;  // row 0 of plane 0
        q.S.qs = q.plane;
        f32::set_copy(a, q.plane, q.S.df, q.S.dg, q.S.phi, q.S.aux);
        f32::set_copy(a + f32::PL_N * q.plane, q.plane, q.S.odf, q.S.odg, q.S.ophi, q.S.oaux);
        q.S.init = a + 2 * f32::PL_N * q.plane;
        q.S.gphi = q.arena + (2 * f32::PL_N + f32::I_N) * q.plane;
    }
    cudaSetDevice(dev0);
    *out = s;
    return DUGKS_OK;
}

extern "C" int dugks_slabs_init(dugks_slabs_t *s, int kind, const double *params, int nparams, uint64_t seed) {
    if (!s) return fail("null handle");
    double iM[16][16] = {};
    std::vector<double> f, h, aux;
    if (host_init_state(s->P, iM, kind, params, nparams, seed, f, h, aux) != DUGKS_OK)
        return fail("unknown init kind for this model");
    const int nx = s->grid.nx, ny = s->grid.ny, pitch = s->P.pitch;
    const size_t n = (size_t)nx * ny;
    // the phase field in the storage layout: g_q = h_q - w_q phi (q = 1..8) and phi
    // = sum_q h_q as the pair (head, tail) of its FP32 rounding
    std::vector<double> g(8 * n), phi2(2 * n);
    for (size_t c = 0; c < n; ++c) {
        double ph = 0.0;
        for (int q = 0; q < 9; ++q) ph += h[(size_t)q * n + c];
        for (int q = 1; q < 9; ++q) g[(size_t)(q - 1) * n + c] = h[(size_t)q * n + c] - d2q9_w(q) * ph;
        const double hi = (double)(float)ph;
        phi2[c] = hi;
        phi2[n + c] = ph - hi;
    }
    const int isrc[f32::I_N] = {F_PHI, F_RHO, F_U, F_V, F_P, F_TAU, F_PHIX, F_PHIY, F_RHOX, F_RHOY, F_FX, F_FY};
    const int asrc[f32::A_N] = {F_FX, F_FY, F_RHOX, F_RHOY, F_PPU, F_PPV};
    for (auto &q : s->parts) {
        cudaSetDevice(q.device);
        const int rows = q.nrows + 2 * H;
        // the partition's rows with halos (periodic wrap; rows outside a walled grid stay 0)
        std::vector<double> tmp((size_t)rows * nx);
        double *stage = nullptr;
        cudaError_t e = cudaMalloc(&stage, tmp.size() * sizeof(double));
        if (e != cudaSuccess) return cuda_fail(e, "init staging");
        auto put = [&](float *plane_row0, const double *src_plane, double sub) -> cudaError_t {
            for (int r = 0; r < rows; ++r) {
                int gj = q.row0 - H + r;
                if (!s->grid.y_walls) gj = ((gj % ny) + ny) % ny;
                double *d = tmp.data() + (size_t)r * nx;
                if (gj < 0 || gj >= ny) std::fill(d, d + nx, sub);
                else std::memcpy(d, src_plane + (size_t)gj * nx, nx * sizeof(double));
            }
            cudaError_t r = cudaMemcpyAsync(stage, tmp.data(), tmp.size() * sizeof(double), cudaMemcpyHostToDevice,
                                            q.st);
            if (r != cudaSuccess) return r;
            r = f32::launch_plane_from_f64<float>(plane_row0 - (size_t)H * pitch, pitch, stage, nx, rows, sub, q.st,
                                                  &s->launches);
            if (r != cudaSuccess) return r;
            return cudaStreamSynchronize(q.st);  // tmp is reused
        };
        for (int k = 0; k < 9 && e == cudaSuccess; ++k)
            e = put(q.S.df + (size_t)k * q.plane, f.data() + (size_t)k * n, internal::rest_f(s->P, k));
        for (int k = 0; k < 8 && e == cudaSuccess; ++k) e = put(q.S.dg + (size_t)k * q.plane, g.data() + (size_t)k * n, 0.0);
        for (int k = 0; k < 2 && e == cudaSuccess; ++k)
            e = put(q.S.phi + (size_t)k * q.plane, phi2.data() + (size_t)k * n, 0.0);
        for (int k = 0; k < f32::I_N && e == cudaSuccess; ++k) {
            const double sub = k == f32::I_DPHI ? DUGKS_F32_PHI0 : (k == f32::I_DP ? 1.0 : 0.0);
            e = put(q.S.init + (size_t)k * q.plane, aux.data() + (size_t)isrc[k] * n, sub);
        }
        for (int k = 0; k < f32::A_N && e == cudaSuccess; ++k)
            e = put(q.S.aux + (size_t)k * q.plane, aux.data() + (size_t)asrc[k] * n, 0.0);
        cudaFree(stage);
        if (e != cudaSuccess) return cuda_fail(e, "init upload");
    }
    s->first = 1;
    s->gcur = 0;
    s->steps = 0;
    return DUGKS_OK;
}

extern "C" int dugks_slabs_step(dugks_slabs_t *s, int nsteps) {
    dugks::TraceRange trace("dugks_slabs_step");
    if (!s || nsteps < 0) return fail("bad argument");
    for (int k = 0; k < nsteps; ++k) {
        const uint32_t sn = (uint32_t)s->steps;
        for (auto &q : s->parts) {
            cudaSetDevice(q.device);
            cudaError_t e = f32::launch_stream32(q.P, q.S, s->first, s->gcur, s->gcur ^ 1, q.st, &s->launches, sn,
                                                 nullptr, 0, nullptr);
            if (e != cudaSuccess) return cuda_fail(e, "partition step");
        }
        if (s->multi_device) {  // every partition's step is done before its rows are copied
            cudaError_t e = sync_all(s);
            if (e != cudaSuccess) return cuda_fail(e, "step");
        }
        for (auto &q : s->parts) f32::swap_io(q.S);
        cudaError_t e = exchange(s);
        if (e != cudaSuccess) return cuda_fail(e, "halo exchange");
        if (s->multi_device && (e = sync_all(s)) != cudaSuccess) return cuda_fail(e, "halo exchange");
        s->first = 0;
        s->gcur ^= 1;
        s->steps += 1;
    }
    return DUGKS_OK;
}

extern "C" int dugks_slabs_download(dugks_slabs_t *s, double *rho, double *u, double *v, double *phi, double *p) {
    if (!s) return fail("null handle");
    const int nx = s->grid.nx, pitch = s->P.pitch;
    double *dst[5] = {rho, u, v, p, phi};
    for (auto &q : s->parts) {
        cudaSetDevice(q.device);
        const size_t fp = (size_t)q.nrows * pitch;
        double *F = q.fields;
        f32::launch_macros32(q.P, q.S, F, F + fp, F + 2 * fp, F + 3 * fp, F + 4 * fp, pitch, q.st, &s->launches);
        for (int k = 0; k < 5; ++k) {
            if (!dst[k]) continue;
            cudaError_t e = cudaMemcpy2DAsync(dst[k] + (size_t)q.row0 * nx, nx * sizeof(double), F + k * fp,
                                              pitch * sizeof(double), nx * sizeof(double), q.nrows,
                                              cudaMemcpyDeviceToHost, q.st);
            if (e != cudaSuccess) return cuda_fail(e, "download");
        }
    }
    cudaError_t e = sync_all(s);
    if (e != cudaSuccess) return cuda_fail(e, "download");
    return DUGKS_OK;
}

// Each partition reduces its own rows on its device (the handle's reduction kernel);
// the host adds the partitions' totals in partition order.
extern "C" int dugks_slabs_reduce(dugks_slabs_t *s, dugks_reductions_t *r) {
    if (!s || !r) return fail("null argument");
    const int pitch = s->P.pitch;
    std::vector<double> tot(4 * s->parts.size());
    for (size_t k = 0; k < s->parts.size(); ++k) {
        Part &q = s->parts[k];
        cudaSetDevice(q.device);
        const size_t fp = (size_t)q.nrows * pitch;
        double *F = q.fields;
        f32::launch_macros32(q.P, q.S, F, F + fp, F + 2 * fp, F + 3 * fp, F + 4 * fp, pitch, q.st, &s->launches);
        Params P = s->P;
        P.ny = q.nrows;
        double *rho_last = q.red, *partial = q.red + fp, *out4 = partial + 4 * RED_BLOCKS;
        exact::launch_reduce(P, F, F + 4 * fp, rho_last, partial, RED_BLOCKS, out4, 1, q.st, &s->launches);
        cudaError_t e = cudaMemcpyAsync(&tot[4 * k], out4, 4 * sizeof(double), cudaMemcpyDeviceToHost, q.st);
        if (e != cudaSuccess) return cuda_fail(e, "reduce");
    }
    cudaError_t e = sync_all(s);
    if (e != cudaSuccess) return cuda_fail(e, "reduce");
    double a = 0, b = 0, d = 0, r2 = 0;
    for (size_t k = 0; k < s->parts.size(); ++k) {
        a += tot[4 * k];
        b += tot[4 * k + 1];
        d += tot[4 * k + 2];
        r2 += tot[4 * k + 3];
    }
    r->sum_rho = a;
    r->sum_phi = b;
    r->residual = std::sqrt(d / (r2 + 1.0E-30));
    r->steps = s->steps;
    return DUGKS_OK;
}

extern "C" int64_t dugks_slabs_launch_count(const dugks_slabs_t *s) { return s ? s->launches : 0; }

extern "C" int dugks_slabs_destroy(dugks_slabs_t *s) {
    if (!s) return DUGKS_OK;
    // partitions of a device share its stream: every partition is done and freed
    // before the streams are destroyed
    for (auto &q : s->parts) {
        cudaSetDevice(q.device);
        if (q.st) cudaStreamSynchronize(q.st);
    }
    for (auto &q : s->parts) {
        cudaSetDevice(q.device);
        if (q.arena) cudaFree(q.arena);
        if (q.fields) cudaFree(q.fields);
        if (q.red) cudaFree(q.red);
    }
    for (auto &q : s->parts) {
        cudaSetDevice(q.device);
        if (q.st && q.own_stream) cudaStreamDestroy(q.st);
    }
    delete s;
    return DUGKS_OK;
}
