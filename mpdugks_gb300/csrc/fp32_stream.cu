// FP32 deviation-storage DUGKS step, streaming form, single case: the kernel
// k_stream32 over the (strip, row segment) items of one grid, its launcher, and the
// tensor map of its TMA row loads.  What a warp does per item is described in
// fp32_stream.cuh; k_stream32 keeps its own copy of that item body, written out in
// the kernel (the shared stream_item, inlined here, gave 4 more registers and a 1.4 %
// slower step on 8192^2 cells), so a change to the per-item steps is made in both:
// tests/test_gpu_serving.py checks the two bit for bit, tests/test_stream_item_copies.py
// that the two texts differ only where they must.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

// constants, ring layouts, TMA helpers shared with the batched streaming kernel
#include "fp32_stream.cuh"

namespace dugks {
namespace f32 {

// first: the first step after an initialisation (the collision takes the state the
// initialisation left instead of the macroscopic quantities of the deviations).  A
// runtime flag, as in the tile kernels, so that both compile the per-cell stages alike
// (the same multiply-add contractions) and give bit-identical results.
// TMA: the stage ring is filled by TMA row loads from `tmap`, a 3-D map (columns,
// rows, planes) over both state copies, the copy a step reads starting at plane
// zin; strips whose window wraps around the periodic x boundary, and slab
// partitions, load per lane with cp.async.  A load not complete within
// TMA_WAIT_LIMIT polls sets *err and ends the warp.
template <int MODEL, bool WALLS, bool TMA>
__global__ void __launch_bounds__(WPB * 32) k_stream32(P32 P, S32 S, int first, int gin, int gout, uint32_t step,
                                                       int nstrips, int nsegs, int seg_rows,
                                                       const __grid_constant__ CUtensorMap tmap, int zin, int *err) {
    using T = float2;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float *wbase = reinterpret_cast<float *>(smem_raw) + (size_t)wib * WARP_F;
    float *stg = wbase;                                   // [NSTG][18][32]
    float *bring = wbase + STG_F;                         // [3] row slots
    float *aring = wbase + STG_F + BR_F;                  // [3] row slots
    auto STG = [&](int slot, int q) -> T {
        return mk2(stg[slot * STG_SLOT + q * 32 + lane], stg[slot * STG_SLOT + (9 + q) * 32 + lane]);
    };
    // mbarriers of this warp's stage slots; their phase parities (bit s: slot s)
    const unsigned bar0 = smem_u32(smem_raw + (size_t)WPB * WARP_F * sizeof(float) + (size_t)wib * NSTG * 8);
    const bool tma_ok = TMA && (smem_u32(smem_raw) & 127u) == 0 && !(P.halo_lo || P.halo_hi);
    uint32_t phases = 0;
    if (TMA) {
        if (lane == 0) {
#pragma unroll
            for (int s = 0; s < NSTG; ++s) mbar_init(bar0 + 8 * s);
            asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        }
        __syncwarp();
    }

    const int nx = P.nx, ny = P.ny, pitch = P.pitch;
    const int gw = blockIdx.x * WPB + wib, nw = gridDim.x * WPB;
    for (int item = gw; item < nstrips * nsegs; item += nw) {
        const int strip = item % nstrips, seg = item / nstrips;
        // the strip's window is columns hs .. hs+31 (a multiple of 4: 16-byte TMA
        // coordinates); its interior columns x0 .. x0+w-1 run over 2 .. nx+1, the
        // last strip's wrapping around the periodic x boundary
        const int hs = strip * SW, x0 = hs + 2, w = min(SW, nx + 2 - x0);
        const int y0 = seg * seg_rows, y1 = min(y0 + seg_rows, ny);
        const int gi = wrap_any(hs + lane, nx);
        const bool use_tma = tma_ok && hs + 32 <= nx;
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
        auto row_of = [&](int j) { return WALLS ? j : (j < 0 ? j + ny : (j >= ny ? j - ny : j)); };
        auto cell = [&](int j) -> long long {  // signed: halo rows lie below row 0
            return (long long)row_of(j) * pitch + gi;
        };
        // wall sides (no halo)
        const bool wlo = WALLS && !hlo, whi = WALLS && !hhi;
        auto loaded = [&](int j) { return j <= y1 + 1 && row_ok(j); };
        auto prefetch = [&](int j) {
            if (loaded(j)) {
                if (use_tma) {
                    if (lane == 0) {
                        const unsigned bar = bar0 + 8 * m4(j);
                        // the slot's previous row was read by every lane (generic proxy)
                        // before this warp's last __syncwarp
                        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                        mbar_expect_tx(bar, STG_TX_BYTES);
                        tma_load_row(smem_u32(stg + m4(j) * STG_SLOT), &tmap, hs, row_of(j), zin, bar);
                    }
                } else {
                    const long long c = cell(j);
                    float *d = stg + m4(j) * STG_SLOT + lane;
#pragma unroll
                    for (int q = 0; q < 9; ++q) {
                        cp_async(d + q * 32, S.df + (size_t)q * S.qs + c);
                        cp_async(d + (9 + q) * 32, S.dh + (size_t)q * S.qs + c);
                    }
                }
            }
            if (!use_tma) cp_async_commit();
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
            const BRow Bm{bring + m3(k - 1) * BR_SLOT}, B0{bring + m3(k) * BR_SLOT}, Bp{bring + m3(k + 1) * BR_SLOT};
            const ARow Am{aring + m3(k - 1) * AR_SLOT}, A0{aring + m3(k) * AR_SLOT}, Ap{aring + m3(k + 1) * AR_SLOT};
            // aux of row k+2, read directly one row ahead of its collision
            const bool coll = k + 1 >= y0 - 1 && row_ok(k + 1) && colL;
            float a6n[A_N];
            if (MODEL != AC && !first && k + 2 >= y0 - 1 && row_ok(k + 2) && colL) {
                const long long c2 = cell(k + 2);
#pragma unroll
                for (int a = 0; a < A_N; ++a) a6n[a] = __ldg(S.aux + (size_t)a * S.qs + c2);
            }
            // row k+2's raw deviations (issued one row ago) have landed
            if (use_tma) {
                if (loaded(k + 2)) {
                    const int s = m4(k + 2);
                    const bool ok = __all_sync(0xffffffffu, mbar_wait(bar0 + 8 * s, (phases >> s) & 1u));
                    if (!ok) {
                        if (lane == 0 && err) atomicExch(err, 1);
                        mbar_wait(bar0 + 8 * s, (phases >> s) & 1u);  // the copy in flight, once more
                        return;
                    }
                    phases ^= 1u << s;
                }
            } else {
                cp_async_wait_all();
            }
            __syncwarp();
            // ---- phi of row k+2
            float sfz2 = 0.f, dph2 = 0.f;
            {
                const int j = k + 2;
                float phv = 0.f;
                if (row_ok(j)) {
                    const int sl = m4(j);
                    T za[9];
#pragma unroll
                    for (int q = 0; q < 9; ++q) za[q] = STG(sl, q);
                    if (MODEL == AC) za[0].x = 0.f;
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
                    for (int q = 0; q < 9; ++q) Pq[q] = STG(sl, q);
                    const float ph[8] = {E, W, ph2, ph0, NE, NW, SE, SWv};
                    const long long c = cell(j);
                    float src[6], phi, U, V;
                    collide_cell<MODEL, float>(P, S, c, first, Pq, sfz1, dph1, a6c, ph, inc_nx, src, phi, U, V);
                    T bp[9];
#pragma unroll
                    for (int q = 0; q < 9; ++q) bp[q] = add2(Pq[q], inc_nx[q]);
                    Bp.put(bp, lane);
                    Ap.put(src, lane);
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
                const BRow &Bg = k == 0 ? Bm : Bp, &B1 = k == 0 ? Bp : Bm;
                const ARow &Ag = k == 0 ? Am : Ap, &A1 = k == 0 ? Ap : Am;
                const T two = mk2(2.f, 2.f);
                T g[9];
#pragma unroll
                for (int q = 0; q < 9; ++q) g[q] = sub2(mul2(two, B0.get(q, lane)), B1.get(q, lane));
                float a0[6], a1[6], ag[6];
                A0.get(a0, lane);
                A1.get(a1, lane);
#pragma unroll
                for (int a = 0; a < 6; ++a) ag[a] = 2.f * a0[a] - a1[a];
                Bg.put(g, lane);
                Ag.put(ag, lane);
            }
            __syncwarp();
            // ---- y-face between rows k-1 and k at the bottom wall (row 0's south face)
            if (wlo && k == 0 && interior) {
                float av[6], am[6], a0[6];
                Am.get(am, lane);
                A0.get(a0, lane);
#pragma unroll
                for (int a = 0; a < 6; ++a) av[a] = 0.5f * (am[a] + a0[a]);
                face_flux<MODEL, false, float>(
                    P, [&](int q) { return Bm.get(q, lane); }, [&](int q) { return B0.get(q, lane); },
                    [&](int q) {
                        return add2(sub2(B0.get(q, lane - 1), B0.get(q, lane + 1)),
                                    sub2(Bm.get(q, lane - 1), Bm.get(q, lane + 1)));
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
                float av[6], a0[6], ap[6];
                A0.get(a0, lane);
                Ap.get(ap, lane);
#pragma unroll
                for (int a = 0; a < 6; ++a) av[a] = 0.5f * (a0[a] + ap[a]);
                const int wall = top_wall ? 2 : 0;
                face_flux<MODEL, false, float>(
                    P, [&](int q) { return B0.get(q, lane); }, [&](int q) { return Bp.get(q, lane); },
                    [&](int q) {
                        return add2(sub2(Bp.get(q, lane - 1), Bp.get(q, lane + 1)),
                                    sub2(B0.get(q, lane - 1), B0.get(q, lane + 1)));
                    },
                    av, wall, FN);
            }
            // ---- x-faces of row k: the west face of every lane, the east face from the next lane
            const bool upd = k >= y0 && row_ok(k);
            T FW[6];
#pragma unroll
            for (int s = 0; s < 6; ++s) FW[s] = mk2(0.f, 0.f);
            if (upd && xfL) {
                float av[6], aw[6], a0[6];
                A0.get(aw, lane - 1);
                A0.get(a0, lane);
#pragma unroll
                for (int a = 0; a < 6; ++a) av[a] = 0.5f * (aw[a] + a0[a]);
                face_flux<MODEL, true, float>(
                    P, [&](int q) { return B0.get(q, lane - 1); }, [&](int q) { return B0.get(q, lane); },
                    [&](int q) {
                        return add2(sub2(Bp.get(q, lane), Bm.get(q, lane)), sub2(Bp.get(q, lane - 1), Bm.get(q, lane - 1)));
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
                for (int q = 0; q < 9; ++q) Pq[q] = STG(sl, q);
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

// Rows of a strip segment.  The persistent warps take the (strip, segment) items in
// turn, so a step lasts as long as the warps with the most items.  First choice: the
// longest of 128, 64, 32 rows that still gives every resident warp about 4 items (a long
// segment costs fewer warm-up rows).  Where that leaves fewer than 8 rounds of items,
// the last, partly filled round is a large share of the step (measured: 2048^2 in 32-row
// segments, 1.3 rounds, takes 1.28x the time of the best length), and the length is
// searched instead: the fill of the last round, (items / warps) / ceil(items / warps),
// times the share of a segment that is not warm-up, len / (len + 4), is maximised.
int stream_segment_rows(int nstrips, int ny, int warps) {
    int seg = SEG_MAX;
    while (seg > 32 && (long long)nstrips * ((ny + seg - 1) / seg) < 4LL * warps) seg /= 2;
    if ((double)nstrips * ((ny + seg - 1) / seg) >= 8.0 * warps) return seg;
    int best = seg;
    double best_eff = -1.0;
    for (int len = 16; len <= ny; ++len) {
        const int n = (ny + len - 1) / len;
        const double waves = (double)nstrips * n / warps;
        const double eff = waves / std::ceil(waves) * ((double)ny / n / ((double)ny / n + 4.0));
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = len;
        }
    }
    return best;
}

template <int MODEL, bool WALLS, bool TMA>
static cudaError_t stream_prepare() {
    cudaError_t e = cudaFuncSetAttribute(k_stream32<MODEL, WALLS, TMA>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)STREAM_SMEM);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stream32<MODEL, WALLS, TMA>, WPB * 32, STREAM_SMEM);
    if (e != cudaSuccess) return e;
    if (per_sm <= 0) return cudaErrorInvalidConfiguration;
    g_stream_blocks = g_stream_blocks ? min(g_stream_blocks, per_sm) : per_sm;
    return cudaSuccess;
}

template <int MODEL, bool WALLS>
static cudaError_t launch_stream_t(const P32 &P, const S32 &S, int first, int gin, int gout, cudaStream_t st,
                                   uint32_t step, const CUtensorMap *tmap, int zin, int *err, bool *fallback) {
    static bool ready = false;
    if (!ready) {
        cudaError_t e = stream_prepare<MODEL, WALLS, false>();
        if (e != cudaSuccess) return e;
        if ((e = stream_prepare<MODEL, WALLS, true>()) != cudaSuccess) return e;
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
    const int seg = stream_segment_rows(nstrips, P.ny, warps);
    const int nsegs = (P.ny + seg - 1) / seg;
    const int items = nstrips * nsegs;
    const int blocks = min((items + WPB - 1) / WPB, g_stream_nsm * g_stream_blocks);
    if (tmap) {
        k_stream32<MODEL, WALLS, true><<<blocks, WPB * 32, STREAM_SMEM, st>>>(P, S, first, gin, gout, step, nstrips,
                                                                            nsegs, seg, *tmap, zin, err);
    } else {
        CUtensorMap none;
        memset(&none, 0, sizeof none);
        k_stream32<MODEL, WALLS, false><<<blocks, WPB * 32, STREAM_SMEM, st>>>(P, S, first, gin, gout, step, nstrips,
                                                                             nsegs, seg, none, 0, err);
    }
    return cudaGetLastError();
}

cudaError_t launch_step32(const P32 &P, const S32 &S, int first, int gin, int gout, cudaStream_t st,
                          int64_t *launches, uint32_t step);

// tmap: null, or the handle's 3-D tensor map over its two state copies (stream_tensor_map);
// zin: the first plane of the copy this step reads (0 or 24); err: the word a staged
// load that did not complete sets
cudaError_t launch_stream32(const P32 &P, const S32 &S, int first, int gin, int gout, cudaStream_t st,
                            int64_t *launches, uint32_t step, const void *tmap, int zin, int *err) {
    // the row window of a segment wraps at most once: grids of fewer than 8 rows
    // run the tile kernel (same arithmetic, same results)
    if (P.ny < 8) return launch_step32(P, S, first, gin, gout, st, launches, step);
    const CUtensorMap *tm = static_cast<const CUtensorMap *>(tmap);
    cudaError_t e = cudaErrorInvalidValue;
    bool fallback = false;
    switch (P.model * 2 + (P.walls ? 1 : 0)) {
        case AC * 2 + 0: e = launch_stream_t<AC, false>(P, S, first, gin, gout, st, step, tm, zin, err, &fallback); break;
        case AC * 2 + 1: e = launch_stream_t<AC, true>(P, S, first, gin, gout, st, step, tm, zin, err, &fallback); break;
        case HCZ * 2 + 0:
            e = launch_stream_t<HCZ, false>(P, S, first, gin, gout, st, step, tm, zin, err, &fallback);
            break;
        case HCZ * 2 + 1:
            e = launch_stream_t<HCZ, true>(P, S, first, gin, gout, st, step, tm, zin, err, &fallback);
            break;
        default: break;
    }
    if (e == cudaSuccess && fallback) return launch_step32(P, S, first, gin, gout, st, launches, step);
    if (e == cudaSuccess) *launches += 1;
    return e;
}

// A 3-D tensor map (x: nx columns, y: ny rows, z: 48 planes) over the two state
// copies of a single-case FP32 handle: 9 f, 9 h and 6 aux planes each, one plane
// every qs floats from `base`; box {32, 1, 18} (the stage slot of one row).
cudaError_t stream_tensor_map(void *map_out, float *base, int nx, int ny, int pitch, size_t qs) {
    using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static EncodeFn encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorSymbolNotFound;
        encode = reinterpret_cast<EncodeFn>(fn);
    }
    if (nx < 32 || ((uintptr_t)base & 15) || ((size_t)pitch * 4) % 16 || (qs * 4) % 16) return cudaErrorInvalidValue;
    const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, 48};
    const cuuint64_t strides[2] = {(cuuint64_t)pitch * 4, (cuuint64_t)qs * 4};
    const cuuint32_t box[3] = {32, 1, 18};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = encode(static_cast<CUtensorMap *>(map_out), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims,
                              strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace f32
}  // namespace dugks
