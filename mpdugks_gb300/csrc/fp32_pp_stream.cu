// FP32 pseudopotential step (D2Q9PP, D2V16) in one streaming pass: k_pp32_stream.
//
// The multi-pass form (fp32_pp.cu) moves ~0.9 KB per cell-update through device memory
// (f-bar-plus, face reconstructions, face psi, fluxes).  Here each warp marches a strip of
// 26 columns (a 32-column window: three halo columns on each side) along y through a
// segment of rows and keeps everything a row needs from its neighbours on the chip:
// f-bar-plus of three rows, the pass-1 face values of two rows and the stage ring of the
// stored remainders in shared memory; psi, the density, the face psi and the face states
// of the rows around in registers (x-neighbours by shuffle).  Per row k, in order:
//   the load of row k+3's remainders into the stage ring;
//   collision of row k+2 (cell force from the 3x3 stencil of the previous psi) into the
//     f-bar-plus ring;
//   face pass 1 of the x faces of row k+1 and of the y face between rows k+1 and k+2
//     (reconstruction, face moments with the previous face force, face psi);
//   face pass 2 of the x faces of row k and of the y face between rows k and k+1 (face
//     force from the face-psi stencil of the faces around -- all of them computed by pass 1
//     of this or earlier rows: the reference's Jacobi semantics -- equilibrium, source,
//     flux);
//   the update of row k.
// A segment starts four rows early; those rows' results are not written.  The per-cell
// and per-face arithmetic is the multi-pass kernels' (fp32_pp.cuh).  The state is read
// from one copy and written to the other (a segment reads rows its neighbours write).
// Periodic in x and y (the pseudopotential models have no walls).
//
// Measured on the GB300 (D2V16, 1024^2): 2.35 G cell-updates/s against 4.10 for the three
// passes, with the same results bit for bit (the equilibrium by opposite-direction pairs,
// which the two forms share, took both up from 1.86 and 3.72).  A lane holds the row pipeline of 16
// distributions (168 registers when compiled for 5 blocks of 2 warps per SM -- 1.69 G at
// the 215 the compiler takes unbounded, 2.00 G at 128 with spills) and the face moments
// and the equation of state are serial float-float chains, so the ~10 resident warps
// cannot hide their latency; the three passes run 40-80 registers a thread at high
// occupancy and, for all their ~0.9 KB of traffic per cell-update, stay ahead.  The handle
// therefore takes the three-pass step; DUGKS_PP_PASSES=1 selects this one.
#include <cuda_runtime.h>

#include <cstdint>

#include "fp32_pp.cuh"

namespace dugks {
namespace f32 {

constexpr int PSW = 26;          // interior columns of a strip
constexpr int PWPB = 2;          // warps per block
constexpr int PP_SEG_MAX = 128;  // longest segment (rows)

template <int MODEL>
struct PPLayout {
    static constexpr int Q = PPQ<MODEL>::Q;
    static constexpr int STG = 4 * Q * 32;  // stage ring: remainders of rows k .. k+3
    static constexpr int BR = 3 * Q * 32;   // f-bar-plus ring: rows k .. k+2
    static constexpr int FB = 2 * Q * 32;   // pass-1 face values of two rows (x faces; y faces)
    static constexpr int WARP_F = STG + BR + 2 * FB;
    static constexpr size_t SMEM = (size_t)PWPB * WARP_F * sizeof(float);
};

__device__ __forceinline__ int pwrap(int j, int n) { return ((j % n) + n) % n; }
__device__ __forceinline__ float2 shdn2(float2 v) {
    return make_float2(__shfl_down_sync(0xffffffffu, v.x, 1), __shfl_down_sync(0xffffffffu, v.y, 1));
}
__device__ __forceinline__ float2 shup2(float2 v) {
    return make_float2(__shfl_up_sync(0xffffffffu, v.x, 1), __shfl_up_sync(0xffffffffu, v.y, 1));
}
__device__ __forceinline__ double shdnd(double v) { return __shfl_down_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ double shupd(double v) { return __shfl_up_sync(0xffffffffu, v, 1); }

// psi pair and its sign G of a cell or a face
struct PsiG {
    float2 psi;
    float g;
};

template <int MODEL>
__global__ void __launch_bounds__(PWPB * 32, 5)
    k_pp32_stream(PPP P, PPV in, PPV out, float *__restrict__ Fxo, float *__restrict__ Fyo, double *__restrict__ pout,
                  size_t qs, int do_msrc, int nstrips, int nsegs, int seg_rows) {
    using L = PPLayout<MODEL>;
    constexpr int Q = L::Q;
    extern __shared__ __align__(16) float psm[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float *stg = psm + (size_t)wib * L::WARP_F;
    float *bring = stg + L::STG;
    float *xbr = bring + L::BR;
    float *ybr = xbr + L::FB;
    const int nx = P.nx, ny = P.ny, pitch = P.pitch;
    const int gw = blockIdx.x * PWPB + wib, nw = gridDim.x * PWPB;
    for (int item = gw; item < nstrips * nsegs; item += nw) {
        const int strip = item % nstrips, seg = item / nstrips;
        const int y0 = seg * seg_rows, y1 = min(y0 + seg_rows, ny);
        const int hs = strip * PSW, w = min(PSW, nx - hs);
        const int gi = pwrap(hs - 3 + lane, nx);
        // lanes of each stage: the update of interior lanes 3 .. 2+w needs the pass-2
        // x faces of lanes 3 .. 3+w and y faces of 3 .. 2+w, whose face-psi stencils need
        // pass 1 one lane further out, whose reconstruction needs f-bar-plus of one more
        const bool l_upd = lane >= 3 && lane < 3 + w;
        const bool l_x2 = lane >= 3 && lane <= 3 + w;
        const bool l_x1 = lane >= 2 && lane <= 4 + w;
        const bool l_y1 = lane >= 2 && lane <= 3 + w;
        const bool l_col = lane >= 1 && lane <= 4 + w;
        auto cell = [&](int j) { return (size_t)pwrap(j, ny) * pitch + gi; };
        auto ld_psi = [&](int j) -> PsiG {
            const size_t c = cell(j);
            return {make_float2(__ldg(in.psi + c), __ldg(in.psil + c)), __ldg(in.scg + c)};
        };
        auto prefetch = [&](int j) {
            if (j <= y1 + 1) {
                const size_t c = cell(j);
                float *d = stg + (size_t)((j + 8) & 3) * Q * 32 + lane;
#pragma unroll
                for (int q = 0; q < Q; ++q) cp_async(d + q * 32, in.g + (size_t)q * qs + c);
            }
            cp_async_commit();
        };
        auto BRQ = [&](int j, int q, int l) -> float { return bring[((j + 9) % 3) * Q * 32 + q * 32 + l]; };
        __syncwarp();  // the previous item is done with this warp's buffers
        prefetch(y0 - 2);
        // rolling per-lane state
        PsiG ps0 = ld_psi(y0 - 3), ps1 = ld_psi(y0 - 2), psn = ld_psi(y0 - 1), ps2;
        double rm = __ldg(in.rho + cell(y0 - 5)), r0 = __ldg(in.rho + cell(y0 - 4)), r1 = __ldg(in.rho + cell(y0 - 3));
        double rn = __ldg(in.rho + cell(y0 - 2)), r2;
        float2 uvn = make_float2((float)__ldg(in.U + cell(y0 - 2)), (float)__ldg(in.V + cell(y0 - 2))), uv2;
        float2 fc0 = make_float2(0.f, 0.f), fc1 = fc0, fc2 = fc0;  // cell forces of rows k, k+1, k+2
        PPFace xm{}, x0{}, xn{};        // x faces of rows k-1, k (pass 2 now), k+1 (pass 1 now)
        PPFace yf0{}, yf1{}, yfn{};     // y faces k, k+1 (pass 2 now), k+2 (pass 1 now)
        float FS[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) FS[q] = 0.f;
        for (int k = y0 - 4; k < y1; ++k) {
            // ---- rows ahead into registers
            ps2 = psn;
            psn = ld_psi(k + 4);
            r2 = rn;
            rn = __ldg(in.rho + cell(k + 3));
            uv2 = uvn;
            uvn = make_float2((float)__ldg(in.U + cell(k + 3)), (float)__ldg(in.V + cell(k + 3)));
            const size_t cx1 = cell(k + 1), cy1 = cell(k + 2);
            const float2 xfp = make_float2(__ldg(in.xFx + cx1), __ldg(in.xFy + cx1));
            const float2 yfp = make_float2(__ldg(in.yFx + cy1), __ldg(in.yFy + cy1));
            // ---- row k+2's remainders have landed; row k+3's load goes out
            cp_async_wait_all();
            __syncwarp();
            prefetch(k + 3);
            // ---- collision of row k+2
            {
                const int j = k + 2;
                const float2 E = shdn2(ps1.psi), W = shup2(ps1.psi), NE = shdn2(ps2.psi), NW = shup2(ps2.psi);
                const float2 SE = shdn2(ps0.psi), SWv = shup2(ps0.psi);
                if (l_col) {
                    const size_t c = cell(j);
                    float fx, fy;
                    if (do_msrc) {
                        float gx, gy;
                        pp_iso_grad(P, E, W, ps2.psi, ps0.psi, NE, NW, SE, SWv, gx, gy);
                        const float kf = -ps1.g * ps1.psi.x;
                        fx = gx * kf;
                        fy = gy * kf;
                    } else {
                        fx = __ldg(Fxo + c);
                        fy = __ldg(Fyo + c);
                    }
                    fc2 = make_float2(fx, fy);
                    float g[Q], bf[Q];
                    const float *sl = stg + (size_t)((j + 8) & 3) * Q * 32 + lane;
#pragma unroll
                    for (int q = 0; q < Q; ++q) g[q] = sl[q * 32];
                    pp_collide<MODEL>(P, g, (float)r2, uv2.x, uv2.y, fx, fy, bf);
                    float *br = bring + (size_t)((j + 9) % 3) * Q * 32 + lane;
#pragma unroll
                    for (int q = 0; q < Q; ++q) br[q * 32] = bf[q];
                }
            }
            __syncwarp();
            // densities of rows k .. k+2 in the west / east lane
            const double r0w = shupd(r0), r1w = shupd(r1), r2w = shupd(r2);
            const double r1e = shdnd(r1), r2e = shdnd(r2);
            // ---- pass 1: x faces of row k+1 (between lanes l-1 and l)
            {
                const int j = k + 1;
                if (j >= y0 - 1 && j <= y1 && l_x1) {
                    float o[Q], n[Q], tn[Q], to[Q], b[Q];
#pragma unroll
                    for (int q = 0; q < Q; ++q) {
                        o[q] = BRQ(j, q, lane - 1);
                        n[q] = BRQ(j, q, lane);
                        tn[q] = BRQ(j + 1, q, lane) - BRQ(j - 1, q, lane);
                        to[q] = BRQ(j + 1, q, lane - 1) - BRQ(j - 1, q, lane - 1);
                    }
                    const double ravg = 0.5 * (r1w + r1);
                    const double hgx = (double)P.hDt * ((r1w - r1) * (double)P.r_ndx);
                    const double hgy = (double)P.hDt * ((0.5 * ((r2 - r0) + (r2w - r0w))) * (double)P.r_2dy);
                    xn = pp_face1<MODEL, true>(P, o, n, tn, to, ravg, hgx, hgy, xfp.x, xfp.y, b);
                    float *d = xbr + (size_t)(j & 1) * Q * 32 + lane;
#pragma unroll
                    for (int q = 0; q < Q; ++q) d[q * 32] = b[q];
                }
            }
            // ---- pass 1: y face between rows k+1 and k+2
            {
                const int j = k + 2;
                if (j >= y0 - 1 && l_y1) {
                    float o[Q], n[Q], tn[Q], to[Q], b[Q];
#pragma unroll
                    for (int q = 0; q < Q; ++q) {
                        o[q] = BRQ(j - 1, q, lane);
                        n[q] = BRQ(j, q, lane);
                        tn[q] = BRQ(j, q, lane - 1) - BRQ(j, q, lane + 1);
                        to[q] = BRQ(j - 1, q, lane - 1) - BRQ(j - 1, q, lane + 1);
                    }
                    const double ravg = 0.5 * (r1 + r2);
                    const double hgx = (double)P.hDt * ((0.5 * ((r2w - r2e) + (r1w - r1e))) * (double)P.r_n2dx);
                    const double hgy = (double)P.hDt * ((r1 - r2) * (double)P.r_ndy);
                    yfn = pp_face1<MODEL, false>(P, o, n, tn, to, ravg, hgx, hgy, yfp.x, yfp.y, b);
                    float *d = ybr + (size_t)(j & 1) * Q * 32 + lane;
#pragma unroll
                    for (int q = 0; q < Q; ++q) d[q * 32] = b[q];
                }
            }
            // ---- pass 2: x faces of row k
            float FW[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) FW[q] = 0.f;
            {
                const float2 xp0 = make_float2(x0.psi, x0.psil), xpm = make_float2(xm.psi, xm.psil);
                const float2 xpn = make_float2(xn.psi, xn.psil);
                const float2 E = shdn2(xp0), W = shup2(xp0), NE = shdn2(xpn), NW = shup2(xpn);
                const float2 SE = shdn2(xpm), SWv = shup2(xpm);
                if (k >= y0 && l_x2) {
                    float gx, gy;
                    pp_iso_grad(P, E, W, xpn, xpm, NE, NW, SE, SWv, gx, gy);
                    const float kf = -x0.scg * x0.psi;
                    const float Fx = gx * kf, Fy = gy * kf;
                    const size_t c = cell(k);
                    if (l_upd) {
                        out.xFx[c] = Fx;
                        out.xFy[c] = Fy;
                    }
                    const float R = (float)(0.5 * (r0w + r0) + (double)x0.dr);
                    float b[Q];
                    const float *s = xbr + (size_t)(k & 1) * Q * 32 + lane;
#pragma unroll
                    for (int q = 0; q < Q; ++q) b[q] = s[q * 32];
                    pp_face2<MODEL, true>(P, b, R, x0, Fx, Fy, FW);
                }
            }
            float FE[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) FE[q] = __shfl_down_sync(0xffffffffu, FW[q], 1);
            // ---- pass 2: y face between rows k and k+1
            float FN[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) FN[q] = 0.f;
            {
                const float2 yp1 = make_float2(yf1.psi, yf1.psil), yp0 = make_float2(yf0.psi, yf0.psil);
                const float2 ypn = make_float2(yfn.psi, yfn.psil);
                const float2 E = shdn2(yp1), W = shup2(yp1), NE = shdn2(ypn), NW = shup2(ypn);
                const float2 SE = shdn2(yp0), SWv = shup2(yp0);
                if (k + 1 >= y0 && l_upd) {
                    float gx, gy;
                    pp_iso_grad(P, E, W, ypn, yp0, NE, NW, SE, SWv, gx, gy);
                    const float kf = -yf1.scg * yf1.psi;
                    const float Fx = gx * kf, Fy = gy * kf;
                    if (k + 1 < y1) {
                        const size_t c = cell(k + 1);
                        out.yFx[c] = Fx;
                        out.yFy[c] = Fy;
                    }
                    const float R = (float)(0.5 * (r0 + r1) + (double)yf1.dr);
                    float b[Q];
                    const float *s = ybr + (size_t)((k + 1) & 1) * Q * 32 + lane;
#pragma unroll
                    for (int q = 0; q < Q; ++q) b[q] = s[q * 32];
                    pp_face2<MODEL, false>(P, b, R, yf1, Fx, Fy, FN);
                }
            }
            // ---- update of row k
            const double r0e = shdnd(r0);
            if (k >= y0 && l_upd) {
                const size_t c = cell(k);
                const float px = (float)(0.5 * (double)P.dtV * (r0w - r0e));
                const float py = (float)(0.5 * (double)P.dtV * (rm - r1));
                float g[Q], bf[Q];
                const float *sl = stg + (size_t)((k + 8) & 3) * Q * 32 + lane;
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    g[q] = sl[q * 32];
                    bf[q] = BRQ(k, q, lane);
                }
                const PPCell n = pp_update<MODEL>(P, g, bf, FW, FE, FS, FN, r0, px, py, fc0.x, fc0.y);
#pragma unroll
                for (int q = 0; q < Q; ++q) out.g[(size_t)q * qs + c] = g[q];
                out.rho[c] = n.rho;
                out.U[c] = n.U;
                out.V[c] = n.V;
                out.psi[c] = n.psi;
                out.psil[c] = n.psil;
                out.scg[c] = n.scg;
                pout[c] = n.p;
                Fxo[c] = fc0.x;
                Fyo[c] = fc0.y;
            }
            // ---- roll the per-lane state one row up
#pragma unroll
            for (int q = 0; q < Q; ++q) FS[q] = FN[q];
            xm = x0;
            x0 = xn;
            yf0 = yf1;
            yf1 = yfn;
            fc0 = fc1;
            fc1 = fc2;
            rm = r0;
            r0 = r1;
            r1 = r2;
            ps0 = ps1;
            ps1 = ps2;
        }
        cp_async_wait_all();  // nothing in flight into this warp's buffers
    }
}

static int g_pp_nsm = 0, g_pp_blocks[2] = {0, 0};

template <int MODEL>
static cudaError_t pp_stream_t(const PPP &P, const PPV &in, const PPV &out, float *Fx, float *Fy, double *p,
                               size_t qs, int do_msrc, cudaStream_t st) {
    using L = PPLayout<MODEL>;
    int &blocks_per_sm = g_pp_blocks[MODEL == PP16 ? 1 : 0];
    if (!blocks_per_sm) {
        cudaError_t e = cudaFuncSetAttribute(k_pp32_stream<MODEL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)L::SMEM);
        if (e != cudaSuccess) return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_pp32_stream<MODEL>, PWPB * 32,
                                                               L::SMEM)) != cudaSuccess)
            return e;
        if (blocks_per_sm <= 0) return cudaErrorInvalidConfiguration;
        int dev = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&g_pp_nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    }
    const int nstrips = (P.nx + PSW - 1) / PSW, warps = g_pp_nsm * blocks_per_sm * PWPB;
    int seg = PP_SEG_MAX;
    while (seg > 16 && (long long)nstrips * ((P.ny + seg - 1) / seg) < 4LL * warps) seg /= 2;
    const int nsegs = (P.ny + seg - 1) / seg, items = nstrips * nsegs;
    const int blocks = min((items + PWPB - 1) / PWPB, g_pp_nsm * blocks_per_sm);
    k_pp32_stream<MODEL><<<blocks, PWPB * 32, L::SMEM, st>>>(P, in, out, Fx, Fy, p, qs, do_msrc, nstrips, nsegs, seg);
    return cudaGetLastError();
}

// One step of the FP32 pseudopotential state in one pass: reads `in`, writes `out`, the
// cell force and the pressure.  Grids of at least 32 columns and 8 rows.
cudaError_t launch_pp32_stream(const PPP &P, const PPV &in, const PPV &out, float *Fx, float *Fy, double *p,
                               size_t qs, int do_msrc, cudaStream_t st, int64_t *launches) {
    if (P.nx < 32 || P.ny < 8) return cudaErrorInvalidValue;
    cudaError_t e = P.model == PP16 ? pp_stream_t<PP16>(P, in, out, Fx, Fy, p, qs, do_msrc, st)
                                    : pp_stream_t<PP9>(P, in, out, Fx, Fy, p, qs, do_msrc, st);
    if (e == cudaSuccess) *launches += 1;
    return e;
}

}  // namespace f32
}  // namespace dugks
