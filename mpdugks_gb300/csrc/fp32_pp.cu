// FP32 deviation-storage step of the pseudopotential models (D2Q9PP, D2V16).
//
// The reference's face force reads the face psi of the neighbouring faces of
// the same step (Ark/Cpp/PseudoP.cpp:39-46, Jacobi semantics: all face psi
// first, then the face forces), so face pass 1 (reconstruction, face moments, face
// psi) of every face precedes face pass 2 (face force, equilibrium, He-Shan-Doolen
// source, flux) of any.  Three launches: the collision (with the cell force from the
// psi of the previous update), face pass 1, and face pass 2 fused with the update (the
// fluxes of a tile in shared memory; with the cell macros, pressure and psi).
//
// Storage: the density rho in FP64 and f as the FP32 remainders g_q = f_q - e_q rho,
// e_q = eq_q(1, 0, 0) the rest equilibrium per unit density.  At rest f = e rho, so
// the g_q are small (the equilibrium's velocity part and the non-equilibrium part)
// where deviations from one global rest state would span the liquid-vapour density
// difference.  The step carries the e_q rho part in closed form: the collision keeps
// it (sum_q (B - f) = 0), the faces reconstruct it from the FP64 density and work
// relative to e_q times the face average of rho, and the update changes rho by the
// sum of the small face fluxes (the e_q avg(rho) parts cancel: sum_q e_q xi_q = 0)
// and each g_q by small increments.  Moment sums and the equation of state are
// float-float (below).
// (Fusing face pass 2 with the update saved the fluxes' round trip through DRAM, ~0.2 KB
// per cell-update, for 0.8 % of the D2V16 step: the passes are latency- as much as
// bandwidth-bound.  An earlier fusion that recomputed the face reconstruction instead of
// reading it ran slower, and so did fusing the collision with face pass 1 (f-bar-plus of
// a 34x10-cell tile ring in shared memory: 127 registers, two blocks per SM, the ring's
// collisions computed twice; 3.09 against 3.54 G cell-updates/s on D2V16 1024^2).)
#include <cuda_runtime.h>

#include <cstdint>

#include "fp32_pp.cuh"

namespace dugks {
namespace f32 {

// 8-neighbour isotropic gradient of a periodic field given as float-float pairs (hi,
// lo planes), from pair differences (Ark/Lib/GradSchemeBasic.h:153-208)
__device__ __forceinline__ void iso_grad(const PPP &P, const float *__restrict__ a, const float *__restrict__ al,
                                         int i, int j, float &gx, float &gy) {
    const int nx = P.nx, ny = P.ny, pitch = P.pitch;
    const int im = wrapi(i - 1, nx), ip = wrapi(i + 1, nx), jm = wrapi(j - 1, ny), jp = wrapi(j + 1, ny);
    auto at = [&](int jj, int ii) {
        const size_t o = (size_t)jj * pitch + ii;
        return make_float2(a[o], al[o]);
    };
    pp_iso_grad(P, at(j, ip), at(j, im), at(jp, i), at(jm, i), at(jp, ip), at(jp, im), at(jm, ip), at(jm, im), gx, gy);
}

// Collision pre-step: cell force F = -G psi grad psi (Ark/Cpp/PseudoP.cpp:31-38, from the
// previous update's psi) when do_msrc, else the stored force; f-bar-plus remainders.
template <int MODEL>
__global__ void __launch_bounds__(256) k_pp32_collide(PPP P, PPS S, int do_msrc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= P.nx || j >= P.ny) return;
    constexpr int Q = PPQ<MODEL>::Q;
    const size_t c = (size_t)j * P.pitch + i;
    float fx, fy;
    if (do_msrc) {
        float gx, gy;
        iso_grad(P, S.psi, S.psil, i, j, gx, gy);
        const float k = -S.scg[c] * S.psi[c];
        fx = gx * k;
        fy = gy * k;
        S.Fx[c] = fx;
        S.Fy[c] = fy;
    } else {
        fx = S.Fx[c];
        fy = S.Fy[c];
    }
    float g[Q], bf[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) g[q] = S.df[(size_t)q * S.qs + c];
    pp_collide<MODEL>(P, g, (float)S.rho[c], (float)S.U[c], (float)S.V[c], fx, fy, bf);
#pragma unroll
    for (int q = 0; q < Q; ++q) S.bf[(size_t)q * S.qs + c] = bf[q];
}

// Face pass 1 (x faces: blockIdx.z = 0, y faces: 1): half-step reconstruction, face
// moments with the previous face force, face pressure and psi (Ark/Lib/D2Q9PP.cpp:110-136,
// Ark/Cpp/PseudoP.cpp:23-30), stored relative to e_q times the face average of rho.
template <int MODEL>
__global__ void __launch_bounds__(256) k_pp32_faces1(PPP P, PPS S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool xf = blockIdx.z == 0;
    if (i >= P.nx || j >= P.ny) return;
    constexpr int Q = PPQ<MODEL>::Q;
    const int nx = P.nx, ny = P.ny, pitch = P.pitch;
    const int im = wrapi(i - 1, nx), ip = wrapi(i + 1, nx), jm = wrapi(j - 1, ny), jp = wrapi(j + 1, ny);
    const size_t c = (size_t)j * pitch + i;
    auto rh = [&](int jj, int ii) { return S.rho[(size_t)jj * pitch + ii]; };
    float o[Q], n[Q], tn[Q], to[Q], b[Q];
    PPFace f;
    if (xf) {  // between (i-1, j) and (i, j)
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const float *F = S.bf + (size_t)q * S.qs;
            auto at = [&](int jj, int ii) { return F[(size_t)jj * pitch + ii]; };
            o[q] = at(j, im);
            n[q] = at(j, i);
            tn[q] = at(jp, i) - at(jm, i);
            to[q] = at(jp, im) - at(jm, im);
        }
        const double ravg = 0.5 * (rh(j, im) + rh(j, i));
        const double hgx = (double)P.hDt * ((rh(j, im) - rh(j, i)) * (double)P.r_ndx);
        const double hgy =
            (double)P.hDt * ((0.5 * ((rh(jp, i) - rh(jm, i)) + (rh(jp, im) - rh(jm, im)))) * (double)P.r_2dy);
        f = pp_face1<MODEL, true>(P, o, n, tn, to, ravg, hgx, hgy, S.xFx[c], S.xFy[c], b);
    } else {  // between (i, j-1) and (i, j)
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const float *F = S.bf + (size_t)q * S.qs;
            auto at = [&](int jj, int ii) { return F[(size_t)jj * pitch + ii]; };
            o[q] = at(jm, i);
            n[q] = at(j, i);
            tn[q] = at(j, im) - at(j, ip);
            to[q] = at(jm, im) - at(jm, ip);
        }
        const double ravg = 0.5 * (rh(jm, i) + rh(j, i));
        const double hgx =
            (double)P.hDt * ((0.5 * ((rh(j, im) - rh(j, ip)) + (rh(jm, im) - rh(jm, ip)))) * (double)P.r_n2dx);
        const double hgy = (double)P.hDt * ((rh(jm, i) - rh(j, i)) * (double)P.r_ndy);
        f = pp_face1<MODEL, false>(P, o, n, tn, to, ravg, hgx, hgy, S.yFx[c], S.yFy[c], b);
    }
    float *B = xf ? S.xb : S.yb;
#pragma unroll
    for (int q = 0; q < Q; ++q) B[(size_t)q * S.qs + c] = b[q];
    (xf ? S.xpsl : S.ypsl)[c] = f.psil;
    (xf ? S.xr : S.yr)[c] = f.dr;
    (xf ? S.xu : S.yu)[c] = f.U;
    (xf ? S.xv : S.yv)[c] = f.V;
    (xf ? S.xg : S.yg)[c] = f.scg;
    (xf ? S.xps : S.yps)[c] = f.psi;
}

// Face pass 2 of the x face (XF) or y face at (i, j): face force from the face-psi
// stencil (Ark/Cpp/PseudoP.cpp:39-46, Ark/Lib/GradSchemeBasic.h:181-208), stored for the
// next step's face moments when own; equilibrium, source and the fluxes xi.n into out.
template <int MODEL, bool XF>
__device__ __forceinline__ void pp_face2_at(const PPP &P, const PPS &S, int i, int j, bool own,
                                            float (&out)[PPQ<MODEL>::Q]) {
    constexpr int Q = PPQ<MODEL>::Q;
    const size_t c = (size_t)j * P.pitch + i;
    float gx, gy;
    iso_grad(P, XF ? S.xps : S.yps, XF ? S.xpsl : S.ypsl, i, j, gx, gy);
    const float k = -(XF ? S.xg : S.yg)[c] * (XF ? S.xps : S.yps)[c];
    const float Fx = gx * k, Fy = gy * k;
    if (own) {
        (XF ? S.xFx : S.yFx)[c] = Fx;
        (XF ? S.xFy : S.yFy)[c] = Fy;
    }
    PPFace f;
    f.dr = (XF ? S.xr : S.yr)[c];
    f.U = (XF ? S.xu : S.yu)[c];
    f.V = (XF ? S.xv : S.yv)[c];
    const size_t co = XF ? (size_t)j * P.pitch + wrapi(i - 1, P.nx) : (size_t)wrapi(j - 1, P.ny) * P.pitch + i;
    const float R = (float)(0.5 * (S.rho[co] + S.rho[c]) + (double)f.dr);
    const float *__restrict__ B = XF ? S.xb : S.yb;
    float b[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) b[q] = B[(size_t)q * S.qs + c];
    pp_face2<MODEL, XF>(P, b, R, f, Fx, Fy, out);
}

// Face pass 2 and the update (Ark/Cpp/DUGKS2DSolver.cpp:748-792) with the cell macros
// (Ark/Lib/D2Q9PP.cpp:89-109) in one launch: a block of 32x8 threads owns a 32x8-cell tile;
// each thread computes the fluxes of its cell's west and south faces into shared memory,
// 40 threads those of the tile's east column and north row (the next tiles' own faces,
// whose forces those tiles store), and after a block barrier each thread updates its cell
// from the four faces' fluxes, which never reach DRAM:
//   rho_new = rho + drho, drho = dt/V sum_q (net face flux of q),
//   g_q,new = g_q + 4/3 (b_q - g_q) + dt/V (net flux of q)
//             + e_q (xi_q,x px + xi_q,y py) - e_q drho,
// px = dt/V (rho_W - rho_E)/2, py = dt/V (rho_S - rho_N)/2 (the e_q avg(rho) flux
// divergence on unit cells, from the FP64 density); U, V, p, psi from float-float
// sums, rho in FP64.
template <int MODEL>
__global__ void __launch_bounds__(256) k_pp32_faces2u(PPP P, PPS S) {
    constexpr int Q = PPQ<MODEL>::Q;
    __shared__ float xs[Q][8][33];  // x-face fluxes of the tile's rows, columns 0 .. 32
    __shared__ float ys[Q][9][32];  // y-face fluxes of the tile's columns, rows 0 .. 8
    const int tx = threadIdx.x, ty = threadIdx.y, t = ty * 32 + tx;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
    const int w = min(32, P.nx - x0), h = min(8, P.ny - y0);
    const int i = x0 + tx, j = y0 + ty;
    const bool in = tx < w && ty < h;
    float out[Q];
    if (in) {
        pp_face2_at<MODEL, true>(P, S, i, j, true, out);
#pragma unroll
        for (int q = 0; q < Q; ++q) xs[q][ty][tx] = out[q];
        pp_face2_at<MODEL, false>(P, S, i, j, true, out);
#pragma unroll
        for (int q = 0; q < Q; ++q) ys[q][ty][tx] = out[q];
    }
    if (t < h) {  // x faces east of the tile (column x0 + w, periodic)
        pp_face2_at<MODEL, true>(P, S, wrapi(x0 + w, P.nx), y0 + t, false, out);
#pragma unroll
        for (int q = 0; q < Q; ++q) xs[q][t][w] = out[q];
    } else if (t >= 32 && t < 32 + w) {  // y faces north of the tile (row y0 + h, periodic)
        pp_face2_at<MODEL, false>(P, S, x0 + t - 32, wrapi(y0 + h, P.ny), false, out);
#pragma unroll
        for (int q = 0; q < Q; ++q) ys[q][h][t - 32] = out[q];
    }
    __syncthreads();
    if (!in) return;
    const int pitch = P.pitch;
    const int ip = wrapi(i + 1, P.nx), im = wrapi(i - 1, P.nx), jn = wrapi(j + 1, P.ny), js = wrapi(j - 1, P.ny);
    const size_t c = (size_t)j * pitch + i;
    const float px = (float)(0.5 * (double)P.dtV * (S.rho[(size_t)j * pitch + im] - S.rho[(size_t)j * pitch + ip]));
    const float py = (float)(0.5 * (double)P.dtV * (S.rho[(size_t)js * pitch + i] - S.rho[(size_t)jn * pitch + i]));
    float g[Q], bf[Q], fw[Q], fe[Q], fs[Q], fn[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const size_t o = (size_t)q * S.qs;
        g[q] = S.df[o + c];
        bf[q] = S.bf[o + c];
        fw[q] = xs[q][ty][tx];
        fe[q] = xs[q][ty][tx + 1];
        fs[q] = ys[q][ty][tx];
        fn[q] = ys[q][ty + 1][tx];
    }
    const PPCell n = pp_update<MODEL>(P, g, bf, fw, fe, fs, fn, S.rho[c], px, py, S.Fx[c], S.Fy[c]);
#pragma unroll
    for (int q = 0; q < Q; ++q) S.df[(size_t)q * S.qs + c] = g[q];
    S.rho_o[c] = n.rho;
    S.psil[c] = n.psil;
    S.U[c] = n.U;
    S.V[c] = n.V;
    S.p[c] = n.p;
    S.scg[c] = n.scg;
    S.psi[c] = n.psi;
}

// One FP64 distribution plane f_q [ny][nx] (dense, as the C ABI passes it) as the
// stored remainder g_q = f_q - e_q rho, rho the FP64 density [ny][pitch]
__global__ void __launch_bounds__(256) k_pp_g_from_f64(float *g, int pitch, const double *__restrict__ f,
                                                       const double *__restrict__ rho, int nx, int ny, double e) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= nx || j >= ny) return;
    const size_t d = (size_t)j * pitch + i;
    g[d] = (float)__dsub_rn(f[(size_t)j * nx + i], __dmul_rn(e, rho[d]));
}

cudaError_t launch_pp_g_from_f64(float *g, int pitch, const double *f, const double *rho, int nx, int ny, double e,
                                 cudaStream_t st, int64_t *launches) {
    const dim3 grd((nx + 255) / 256, ny);
    k_pp_g_from_f64<<<grd, 256, 0, st>>>(g, pitch, f, rho, nx, ny, e);
    *launches += 1;
    return cudaGetLastError();
}

// the cell force of the current psi (the state the reference holds after a step)
__global__ void __launch_bounds__(256) k_pp32_force(PPP P, PPS S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= P.nx || j >= P.ny) return;
    const size_t c = (size_t)j * P.pitch + i;
    float gx, gy;
    iso_grad(P, S.psi, S.psil, i, j, gx, gy);
    const float k = -S.scg[c] * S.psi[c];
    S.Fx[c] = gx * k;
    S.Fy[c] = gy * k;
}

template <int MODEL>
static cudaError_t launch_pp_t(const PPP &P, const PPS &S, int do_msrc, cudaStream_t st, int64_t *launches,
                               uint32_t step) {
    const dim3 blk(32, 8);
    const dim3 grd((P.nx + 31) / 32, (P.ny + 7) / 8), grf(grd.x, grd.y, 2);
    (void)step;
    k_pp32_collide<MODEL><<<grd, blk, 0, st>>>(P, S, do_msrc);
    k_pp32_faces1<MODEL><<<grf, blk, 0, st>>>(P, S);
    k_pp32_faces2u<MODEL><<<grd, blk, 0, st>>>(P, S);
    *launches += 3;
    return cudaGetLastError();
}

cudaError_t launch_pp32_step(const PPP &P, const PPS &S, int do_msrc, cudaStream_t st, int64_t *launches,
                             uint32_t step) {
    return P.model == PP16 ? launch_pp_t<PP16>(P, S, do_msrc, st, launches, step)
                           : launch_pp_t<PP9>(P, S, do_msrc, st, launches, step);
}

cudaError_t launch_pp32_force(const PPP &P, const PPS &S, cudaStream_t st, int64_t *launches) {
    const dim3 blk(32, 8);
    const dim3 grd((P.nx + 31) / 32, (P.ny + 7) / 8);
    k_pp32_force<<<grd, blk, 0, st>>>(P, S);
    *launches += 1;
    return cudaGetLastError();
}

}  // namespace f32
}  // namespace dugks
