// FP32 deviation-storage DUGKS step, streaming form: one warp per strip of
// 28 columns (plus a two-column halo on each side, 32 lanes), marching along
// y through a segment of rows.  No block-wide barrier: the y-neighbours of a
// row are in the warp's own rolling buffers (shared memory), the
// x-neighbours are the adjacent lanes' entries of the same buffers (or a
// shuffle), so every warp runs independently of the others and of its block.
//
// Per row k the warp does, in order:
//   phi of row k+2 (float-float sum of its h deviations, staged in shared
//     memory); cp.async of row k+3's deviations into the stage ring (the
//     aux of a row is read directly into registers one row ahead of its
//     collision);
//   collision of row k+1 (macros, MacroSource on the 3x3 phi stencil from
//     the phi of rows k..k+2 and the adjacent lanes, f-bar-plus) into the
//     f-bar-plus ring;
//   the y-face between rows k and k+1 (its flux is row k's north face and,
//     carried to the next row, row k+1's south face);
//   the x-faces of row k (west face per lane, east face from the next lane);
//   the update of row k.
// A segment starts four rows early (phi of rows y0-2 and y0-1, collision of
// row y0-1, the face below row y0); those rows' results are not written.
// Bounce-back walls: ghost rows -1 and ny of f-bar-plus and of the averaged
// fields are extrapolated (2 a0 - a1) into the rings and the wall faces bounce
// back, as in the tile kernel.  The per-cell arithmetic is the tile kernel's
// (fp32_math.cuh) with the same random bits, so the two kernels give
// bit-identical results.
#include <cuda_runtime.h>

#include <cstdint>

#include "dugks_device.cuh"
#include "fp32_math.cuh"
#include "fp32_state.cuh"

namespace dugks {
namespace f32 {

constexpr int SW = 28;   // interior columns of a strip
constexpr int SEG_MAX = 128;  // rows of a segment: 128, 64 or 32 (enough segments per warp)
constexpr int WPB = 2;   // warps per block
constexpr int NSTG = 4;  // stage ring: rows k .. k+3
constexpr int NPL = 18;  // staged planes per row: f and h deviations (aux is read directly)
// per-warp shared memory (floats): stage ring [NSTG][18][32], f-bar-plus ring
// [3][9][32] pairs, averaged-field ring [3][6][32]
constexpr int STG_F = NSTG * NPL * 32;
constexpr int BR_F = 3 * 9 * 32 * 2;
constexpr int AR_F = 3 * 6 * 32;
constexpr int WARP_F = STG_F + BR_F + AR_F;
constexpr size_t STREAM_SMEM = (size_t)WPB * WARP_F * sizeof(float);

__device__ __forceinline__ int m3(int j) { return (j + 6) % 3; }  // j >= -6
__device__ __forceinline__ int m4(int j) { return (j + 8) & 3; }  // j >= -8
__device__ __forceinline__ int wrap_any(int j, int n) { return ((j % n) + n) % n; }

template <int MODEL, bool WALLS>
__global__ void __launch_bounds__(WPB * 32) k_stream32(P32 P, S32 S, int first, int gin, int gout, uint32_t step,
                                                       int nstrips, int nsegs, int seg_rows) {
    using T = float2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float *wbase = reinterpret_cast<float *>(smem_raw) + (size_t)wib * WARP_F;
    float *stg = wbase;                                   // [NSTG][NPL][32]
    T *bring = reinterpret_cast<T *>(wbase + STG_F);      // [3][9][32]
    float *aring = wbase + STG_F + BR_F;                  // [3][6][32]
    auto STG = [&](int slot, int p) -> float & { return stg[(slot * NPL + p) * 32 + lane]; };

    const int nx = P.nx, ny = P.ny, pitch = P.pitch;
    const int gw = blockIdx.x * WPB + wib, nw = gridDim.x * WPB;
    for (int item = gw; item < nstrips * nsegs; item += nw) {
        const int strip = item % nstrips, seg = item / nstrips;
        const int x0 = strip * SW, w = min(SW, nx - x0);
        const int y0 = seg * seg_rows, y1 = min(y0 + seg_rows, ny);
        const int gi = wrap_any(x0 - 2 + lane, nx);
        const bool interior = lane >= 2 && lane < 2 + w;
        const bool colL = lane >= 1 && lane <= 2 + w;  // lanes whose f-bar-plus is needed
        const bool xfL = lane >= 2 && lane <= 2 + w;   // lanes whose west x-face is needed
        // rows of the window lie in [y0-4, y1+3] (the launcher ensures ny >= 8).  A
        // slab partition (WALLS instance) reads rows below 0 / from ny up from its
        // halo rows where halo_lo / halo_hi is set; elsewhere they are walls.
        const bool hlo = WALLS && P.halo_lo, hhi = WALLS && P.halo_hi;
        auto row_ok = [&](int j) {
            return WALLS ? ((j >= 0 || (hlo && j >= -SLAB_HALO)) && (j < ny || (hhi && j < ny + SLAB_HALO))) : true;
        };
        auto cell = [&](int j) -> long long {  // signed: halo rows lie below row 0
            const int jj = WALLS ? j : (j < 0 ? j + ny : (j >= ny ? j - ny : j));
            return (long long)jj * pitch + gi;
        };
        // wall sides (no halo)
        const bool wlo = WALLS && !hlo, whi = WALLS && !hhi;
        auto prefetch = [&](int j) {
            if (j <= y1 + 1 && row_ok(j)) {
                const long long c = cell(j);
                float *d = stg + m4(j) * NPL * 32 + lane;
#pragma unroll
                for (int q = 0; q < 9; ++q) {
                    cp_async(d + q * 32, S.df + (size_t)q * S.qs + c);
                    cp_async(d + (9 + q) * 32, S.dh + (size_t)q * S.qs + c);
                }
            }
            cp_async_commit();
        };
        __syncwarp();  // the previous item is done with this warp's buffers
        prefetch(y0 - 2);
        // rolling per-lane state: phi of rows k, k+1, k+2; the (sum f, sum h)
        // deviation sums of rows k+1, k+2; row k's collision increments and
        // south-face flux
        float ph0 = 0.f, ph1 = 0.f, ph2 = 0.f;
        float sfz1 = 0.f, dph1 = 0.f;
        float a6c[A_N];  // aux of row k+1 (loaded at the previous row)
        T inc_cur[9], FS[6];
#pragma unroll
        for (int q = 0; q < 9; ++q) inc_cur[q] = mk2(0.f, 0.f);
#pragma unroll
        for (int s = 0; s < 6; ++s) FS[s] = mk2(0.f, 0.f);
        for (int k = y0 - 4; k < y1; ++k) {
            // this row's ring slots: f-bar-plus and averaged fields of rows k-1, k, k+1
            T *const Bm = bring + m3(k - 1) * 288, *const B0 = bring + m3(k) * 288, *const Bp = bring + m3(k + 1) * 288;
            float *const Am = aring + m3(k - 1) * 192, *const A0 = aring + m3(k) * 192,
                         *const Ap = aring + m3(k + 1) * 192;
            // aux of row k+2, read directly one row ahead of its collision
            const bool coll = k + 1 >= y0 - 1 && row_ok(k + 1) && colL;
            float a6n[A_N];
            if (MODEL != AC && !first && k + 2 >= y0 - 1 && row_ok(k + 2) && colL) {
                const long long c2 = cell(k + 2);
#pragma unroll
                for (int a = 0; a < A_N; ++a) a6n[a] = __ldg(S.aux + (size_t)a * S.qs + c2);
            }
            cp_async_wait_all();
            __syncwarp();
            // ---- phi of row k+2
            float sfz2 = 0.f, dph2 = 0.f;
            {
                const int j = k + 2;
                float phv = 0.f;
                if (row_ok(j)) {
                    const int sl = m4(j);
                    T za[9];
                    za[0] = mk2(MODEL == AC ? 0.f : STG(sl, 0), STG(sl, 9));
#pragma unroll
                    for (int q = 1; q < 9; ++q) za[q] = mk2(STG(sl, q), STG(sl, 9 + q));
                    const T z = ff_sum9(za);
                    sfz2 = z.x;
                    dph2 = z.y;
                    phv = P.phi0 + dph2;
                } else if ((wlo && j == -1) || (whi && j == ny)) {
                    // ghost phi: the previous step's extrapolation (Ark/Cpp/Boundary.cpp:38-63)
                    phv = S.gphi[(size_t)(gin * 2 + (j < 0 ? 0 : 1)) * pitch + gi];
                }
                ph2 = phv;
            }
            __syncwarp();  // every lane has read slot k+2 (slot k+3 = slot k-1 is refilled next)
            prefetch(k + 3);
            // ---- collision of row k+1
            T inc_nx[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) inc_nx[q] = mk2(0.f, 0.f);
            {
                const int j = k + 1;
                // 3x3 phi stencil: rows k (S), k+1, k+2 (N); lanes +-1 (E/W)
                const float E = __shfl_down_sync(0xffffffffu, ph1, 1), W = __shfl_up_sync(0xffffffffu, ph1, 1);
                const float NE = __shfl_down_sync(0xffffffffu, ph2, 1), NW = __shfl_up_sync(0xffffffffu, ph2, 1);
                const float SE = __shfl_down_sync(0xffffffffu, ph0, 1), SWv = __shfl_up_sync(0xffffffffu, ph0, 1);
                if (coll) {
                    const int sl = m4(j);
                    T Pq[9];
#pragma unroll
                    for (int q = 0; q < 9; ++q) Pq[q] = mk2(STG(sl, q), STG(sl, 9 + q));
                    const float ph[8] = {E, W, ph2, ph0, NE, NW, SE, SWv};
                    const long long c = cell(j);
                    float src[6], phi, U, V;
                    collide_cell<MODEL, float>(P, S, c, first, Pq, sfz1, dph1, a6c, ph, inc_nx, src, phi, U, V);
#pragma unroll
                    for (int q = 0; q < 9; ++q) Bp[q * 32 + lane] = add2(Pq[q], inc_nx[q]);
#pragma unroll
                    for (int a = 0; a < 6; ++a) Ap[a * 32 + lane] = src[a];
                    if (j >= y0 && j < y1 && interior) {
                        if (MODEL != AC) {
                            S.oaux[A_FX * S.qs + c] = src[4];
                            S.oaux[A_FY * S.qs + c] = src[5];
                            S.oaux[A_RHOX * S.qs + c] = src[2];
                            S.oaux[A_RHOY * S.qs + c] = src[3];
                            S.oaux[A_PPU * S.qs + c] = phi * U;
                            S.oaux[A_PPV * S.qs + c] = phi * V;
                        }
                        // ghost phi for the next step's MacroSource
                        if (wlo && j == 0) S.gphi[(size_t)(gout * 2 + 0) * pitch + gi] = 2.f * phi - ph2;
                        if (whi && j == ny - 1) S.gphi[(size_t)(gout * 2 + 1) * pitch + gi] = 2.f * phi - ph0;
                    }
                }
            }
            __syncwarp();
            // ---- wall ghost rows of f-bar-plus and of the averaged fields (2 a0 - a1)
            if (((wlo && k == 0) || (whi && k == ny - 1)) && colL) {
                // bottom: row -1 (slot of k-1) from rows 0 (k), 1 (k+1); top: row ny (slot of
                // k+1) from rows ny-1 (k), ny-2 (k-1)
                T *const Bg = k == 0 ? Bm : Bp, *const B1 = k == 0 ? Bp : Bm;
                float *const Ag = k == 0 ? Am : Ap, *const A1 = k == 0 ? Ap : Am;
                const T two = mk2(2.f, 2.f);
#pragma unroll
                for (int q = 0; q < 9; ++q) Bg[q * 32 + lane] = sub2(mul2(two, B0[q * 32 + lane]), B1[q * 32 + lane]);
#pragma unroll
                for (int a = 0; a < 6; ++a) Ag[a * 32 + lane] = 2.f * A0[a * 32 + lane] - A1[a * 32 + lane];
            }
            __syncwarp();
            // ---- y-face between rows k-1 and k at the bottom wall (row 0's south face)
            if (wlo && k == 0 && interior) {
                float av[6];
#pragma unroll
                for (int a = 0; a < 6; ++a) av[a] = 0.5f * (Am[a * 32 + lane] + A0[a * 32 + lane]);
                face_flux<MODEL, false, float>(
                    P, [&](int q) { return Bm[q * 32 + lane]; }, [&](int q) { return B0[q * 32 + lane]; },
                    [&](int q) {
                        return add2(sub2(B0[q * 32 + lane - 1], B0[q * 32 + lane + 1]),
                                    sub2(Bm[q * 32 + lane - 1], Bm[q * 32 + lane + 1]));
                    },
                    av, 1, FS);
            }
            // ---- y-face between rows k and k+1 (row k's north face)
            T FN[6];
#pragma unroll
            for (int s = 0; s < 6; ++s) FN[s] = mk2(0.f, 0.f);
            const bool top_wall = whi && k == ny - 1;
            const bool yface = k >= y0 - 1 && ((row_ok(k) && row_ok(k + 1)) || top_wall);
            if (yface && interior) {
                float av[6];
#pragma unroll
                for (int a = 0; a < 6; ++a) av[a] = 0.5f * (A0[a * 32 + lane] + Ap[a * 32 + lane]);
                const int wall = top_wall ? 2 : 0;
                face_flux<MODEL, false, float>(
                    P, [&](int q) { return B0[q * 32 + lane]; }, [&](int q) { return Bp[q * 32 + lane]; },
                    [&](int q) {
                        return add2(sub2(Bp[q * 32 + lane - 1], Bp[q * 32 + lane + 1]),
                                    sub2(B0[q * 32 + lane - 1], B0[q * 32 + lane + 1]));
                    },
                    av, wall, FN);
            }
            // ---- x-faces of row k: the west face of every lane, the east face from the next lane
            const bool upd = k >= y0 && row_ok(k);
            T FW[6];
#pragma unroll
            for (int s = 0; s < 6; ++s) FW[s] = mk2(0.f, 0.f);
            if (upd && xfL) {
                float av[6];
#pragma unroll
                for (int a = 0; a < 6; ++a) av[a] = 0.5f * (A0[a * 32 + lane - 1] + A0[a * 32 + lane]);
                face_flux<MODEL, true, float>(
                    P, [&](int q) { return B0[q * 32 + lane - 1]; }, [&](int q) { return B0[q * 32 + lane]; },
                    [&](int q) {
                        return add2(sub2(Bp[q * 32 + lane], Bm[q * 32 + lane]),
                                    sub2(Bp[q * 32 + lane - 1], Bm[q * 32 + lane - 1]));
                    },
                    av, 0, FW);
            }
            T FE[6];
#pragma unroll
            for (int s = 0; s < 6; ++s)
                FE[s] = mk2(__shfl_down_sync(0xffffffffu, FW[s].x, 1), __shfl_down_sync(0xffffffffu, FW[s].y, 1));
            // ---- update of row k
            if (upd && interior) {
                const int sl = m4(k);
                T Pq[9], dn[9];
#pragma unroll
                for (int q = 0; q < 9; ++q) Pq[q] = mk2(STG(sl, q), STG(sl, 9 + q));
                const long long c = cell(k);
                update_cell<float>(P, Pq, inc_cur, FW, FE, FS, FN, sr_bits(P, k, gi, step), dn);
#pragma unroll
                for (int q = 0; q < 9; ++q) {
                    S.odf[(size_t)q * S.qs + c] = dn[q].x;
                    S.odh[(size_t)q * S.qs + c] = dn[q].y;
                }
            }
            // ---- roll the per-lane state one row up
#pragma unroll
            for (int q = 0; q < 9; ++q) inc_cur[q] = inc_nx[q];
#pragma unroll
            for (int s = 0; s < 6; ++s) FS[s] = FN[s];
            ph0 = ph1;
            ph1 = ph2;
            sfz1 = sfz2;
            dph1 = dph2;
            if (MODEL != AC) {
#pragma unroll
                for (int a = 0; a < A_N; ++a) a6c[a] = a6n[a];
            }
        }
        cp_async_wait_all();  // nothing in flight into this warp's buffers
    }
}

static int g_stream_nsm = 0, g_stream_blocks = 0;

template <int MODEL, bool WALLS>
static cudaError_t stream_prepare() {
    cudaError_t e = cudaFuncSetAttribute(k_stream32<MODEL, WALLS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)STREAM_SMEM);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stream32<MODEL, WALLS>, WPB * 32, STREAM_SMEM);
    if (e != cudaSuccess) return e;
    if (per_sm <= 0) return cudaErrorInvalidConfiguration;
    g_stream_blocks = g_stream_blocks ? min(g_stream_blocks, per_sm) : per_sm;
    return cudaSuccess;
}

template <int MODEL, bool WALLS>
static cudaError_t launch_stream_t(const P32 &P, const S32 &S, int first, int gin, int gout, cudaStream_t st,
                                   uint32_t step, bool *fallback) {
    static bool ready = false;
    if (!ready) {
        cudaError_t e = stream_prepare<MODEL, WALLS>();
        if (e != cudaSuccess) return e;
        int dev = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&g_stream_nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        ready = true;
    }
    // the longest segment that still gives every resident warp about 4 segments
    // (a long segment costs fewer warm-up rows, a short one less idle tail)
    const int nstrips = (P.nx + SW - 1) / SW, warps = g_stream_nsm * g_stream_blocks * WPB;
    // a grid with fewer 32-row strip segments than resident warps leaves most of the
    // GPU idle in this form: the tile kernel (same arithmetic, same results) runs it
    // (a slab partition reads halo rows, which only this form does: it always runs here)
    if (!(P.halo_lo || P.halo_hi) && (long long)nstrips * ((P.ny + 31) / 32) < warps) {
        *fallback = true;
        return cudaSuccess;
    }
    int seg = SEG_MAX;
    while (seg > 32 && (long long)nstrips * ((P.ny + seg - 1) / seg) < 4LL * warps) seg /= 2;
    const int nsegs = (P.ny + seg - 1) / seg;
    const int items = nstrips * nsegs;
    const int blocks = min((items + WPB - 1) / WPB, g_stream_nsm * g_stream_blocks);
    k_stream32<MODEL, WALLS><<<blocks, WPB * 32, STREAM_SMEM, st>>>(P, S, first, gin, gout, step, nstrips, nsegs,
                                                                     seg);
    return cudaGetLastError();
}

cudaError_t launch_step32(const P32 &P, const S32 &S, int first, int gin, int gout, cudaStream_t st,
                          int64_t *launches, uint32_t step);

cudaError_t launch_stream32(const P32 &P, const S32 &S, int first, int gin, int gout, cudaStream_t st,
                            int64_t *launches, uint32_t step) {
    // the row window of a segment wraps at most once: grids of fewer than 8 rows
    // run the tile kernel (same arithmetic, same results)
    if (P.ny < 8) return launch_step32(P, S, first, gin, gout, st, launches, step);
    cudaError_t e = cudaErrorInvalidValue;
    bool fallback = false;
    switch (P.model * 2 + (P.walls ? 1 : 0)) {
        case AC * 2 + 0: e = launch_stream_t<AC, false>(P, S, first, gin, gout, st, step, &fallback); break;
        case AC * 2 + 1: e = launch_stream_t<AC, true>(P, S, first, gin, gout, st, step, &fallback); break;
        case HCZ * 2 + 0: e = launch_stream_t<HCZ, false>(P, S, first, gin, gout, st, step, &fallback); break;
        case HCZ * 2 + 1: e = launch_stream_t<HCZ, true>(P, S, first, gin, gout, st, step, &fallback); break;
        default: break;
    }
    if (e == cudaSuccess && fallback) return launch_step32(P, S, first, gin, gout, st, launches, step);
    if (e == cudaSuccess) *launches += 1;
    return e;
}

}  // namespace f32
}  // namespace dugks
