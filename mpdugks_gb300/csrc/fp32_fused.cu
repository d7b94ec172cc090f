// FP32 deviation-storage DUGKS step: one fused kernel per time step.
//
// Storage (fp32_state.cuh): f~ as FP32 deviations from fixed rest equilibria,
//   HCZ: f0_q = w_q p0;  AC: f0_q = w_q p0/RT - [q=0] p0/RT  (p0 = 1);
// h~ as the phase field phi (a float-float pair) and the remainders
// g_q = h_q - w_q phi (q = 1..8) in FP32.  Every step relation of the reference
// is affine with coefficients that sum to one (aBP + bBP = 1, ah + bh = 1,
// 4/3 - 1/3 = 1) and the rest parts of the four face fluxes of a cell cancel
// (sum of +-xi.n = 0, bounce-back maps q to a direction of equal weight), so the
// step is carried out on the deviations directly; the rest moments enter only the
// macroscopic quantities (p = p0 + dp).  The phase field's w_q phi part is carried
// through the step in closed form (fp32_math.cuh): the faces work relative to
// w_q times the face average of phi, phi changes by the sum of the small face
// fluxes, and the g_q by small increments.  Cell moment sums (rho u, rho v, p)
// are float-float (Knuth two-sum) sums of the FP32 deviations; the domain sums
// and residual are FP64 reductions.
//
// One CTA = 32 x 16 threads over a 30 x 14 tile of cells plus a one-cell
// halo ring: every thread owns one cell of the (w+2) x (h+2) region, computes
// its macroscopic quantities, MacroSource (3x3 phi stencil from shared
// memory, halo 2) and f-bar-plus; then its west x-face and south y-face
// (CD reconstruction, face moments, equilibria, flux); the east face comes
// from the next lane by shuffle, the north face from shared memory; interior
// threads then apply the finite-volume update and write their deviations.
// Cells in two tiles' halos are computed by both with the same operation
// order, so shared faces carry bit-identical fluxes and mass is conserved.
// A step reads one copy of the state and writes the other (tiles read their
// neighbours' cells as halo, so an in-place update would race across waves).
//
// Phase references: P1 Ark/Cpp/DUGKS2DSolver.cpp:175-183 (Ark/Lib/D2Q9HCZ.cpp:54-92,
// Ark/Lib/D2Q9AC.cpp:69-105); P4 :219-250 (CD_Interior_phi_Bh :604-687);
// P8 :748-792; P9 Ark/Lib/D2Q9HCZ.cpp:133-182; P10 Ark/Cpp/SourceM.cpp:35-62.
#include <cuda_runtime.h>

#include <cstdint>

#include "dugks_device.cuh"
#include "fp32_state.cuh"
#include "fp32_math.cuh"
#include "fp32_stream.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace dugks {
namespace f32 {

constexpr int TW = 30, TH = 14;  // interior tile
constexpr int BX = 32, BY = 16;  // threads = tile + halo ring


// phi pairs (halo 2), f-bar-plus pairs, south-face flux pairs, averaged fields
constexpr size_t SMEM_ELEMS = (size_t)2 * (BY + 2) * (BX + 2) + (18 + 6 + 12) * BY * BX;
// Prefetch staging (storage type float only): the next tile's own-cell planes
// (the PL_N planes of a state copy) and the phi pairs of its phi ring, copied
// asynchronously (cp.async) while the current tile computes.
constexpr int RING_MAX = 2 * (TW + 4) + 2 * (TH + 2);  // ring cells of a full tile
constexpr size_t STG_ELEMS = (size_t)PL_N * BY * BX + 2 * RING_MAX;
template <typename R>
constexpr bool prefetched() { return sizeof(R) == 4; }
template <typename R>
constexpr size_t smem_elems() { return SMEM_ELEMS + (prefetched<R>() ? STG_ELEMS : 0); }


// Geometry of tile t as seen by thread (e, r): the tile's interior origin and
// size, and this thread's extended cell (interior plus a one-cell ring).
template <bool WALLS>
struct TileCell {
    int x0, y0, w, hh, gi, gj;
    bool act, ghost, real;
    size_t c;
    __device__ __forceinline__ TileCell(int t, int ntx, int e, int r, int nx, int ny, int pitch) {
        x0 = (t % ntx) * TW;
        y0 = (t / ntx) * TH;
        w = min(TW, nx - x0);
        hh = min(TH, ny - y0);
        act = (e <= w + 1) && (r <= hh + 1);
        gi = wrapi(x0 + e - 1, nx);
        gj = y0 + r - 1;
        ghost = false;  // wall ghost row (values extrapolated in shared memory)
        if (WALLS) {
            if (gj < 0 || gj >= ny) ghost = true;
        } else {
            gj = wrapi(gj, ny);
        }
        real = act && !ghost;
        c = real ? (size_t)gj * pitch + gi : 0;
    }
    // ring of the phi region (halo 2): index k in [0, nring) -> (re, rr) in
    // tile coordinates, e in {-1, w+2} or r in {-1, hh+2}
    __device__ __forceinline__ int nring() const { return 2 * (w + 4) + 2 * (hh + 2); }
    __device__ __forceinline__ void ring(int k, int &re, int &rr) const {
        const int RW = w + 4;
        if (k < RW) { re = k - 1; rr = -1; }
        else if (k < 2 * RW) { re = k - RW - 1; rr = hh + 2; }
        else if (k < 2 * RW + hh + 2) { re = -1; rr = k - 2 * RW; }
        else { re = w + 2; rr = k - 2 * RW - (hh + 2); }
    }
};

// Issue the asynchronous copies of tile t's inputs into the staging area.
template <int MODEL, bool WALLS>
__device__ __forceinline__ void prefetch_tile(const PR<float> &P, const SR<float> &S, int t, int ntx, int e, int r,
                                              int tid, float *stg, float *stg_ring) {
    const TileCell<WALLS> g(t, ntx, e, r, P.nx, P.ny, P.pitch);
    if (g.real) {
        float *d = stg + r * BX + e;
        constexpr int BS = BY * BX;
        // f, g, phi; the aux planes only for the flow-solving model (AC: u = 0)
        constexpr int NPL = MODEL == AC ? PL_AUX : PL_N;
#pragma unroll
        for (int k = 0; k < NPL; ++k) cp_async(d + k * BS, S.df + (size_t)k * S.qs + g.c);
    }
    const int nr = g.nring();
    for (int k = tid; k < nr; k += BX * BY) {
        int re, rr;
        g.ring(k, re, rr);
        int rj = g.y0 + rr - 1;
        if (WALLS && (rj < 0 || rj >= P.ny)) continue;  // ghost phi or unused
        if (!WALLS) rj = wrapi(rj, P.ny);
        const size_t cc = (size_t)rj * P.pitch + wrapi(g.x0 + re - 1, P.nx);
        cp_async(stg_ring + k, S.phi + cc);
        cp_async(stg_ring + RING_MAX + k, S.phi + S.qs + cc);
    }
    cp_async_commit();
}

// Shared-memory views of one CTA
template <typename R>
struct Views {
    using T = typename Pair<R>::T;
    T (*sB)[BY][BX];       // f-bar-plus pairs
    T (*sFS)[BY][BX];      // south-face flux pairs (6 slots)
    R (*sA)[BY][BX];       // srcx srcy rhox rhoy fx fy
    T (*sphi)[BX + 2];     // phi pairs (head, tail), halo 2
    R *stg;                // [PL_N][BY][BX] staged own-cell inputs (prefetch)
    R *stg_ring;           // [2][RING_MAX] staged ring phi pairs (prefetch)
    __device__ __forceinline__ explicit Views(unsigned char *raw) {
        R *smem = reinterpret_cast<R *>(raw);
        sB = reinterpret_cast<T(*)[BY][BX]>(smem);
        sFS = sB + 9;
        sA = reinterpret_cast<R(*)[BY][BX]>(sFS + 6);
        sphi = reinterpret_cast<T(*)[BX + 2]>(smem + (18 + 12 + 6) * BY * BX);
        stg = smem + SMEM_ELEMS;
        stg_ring = stg + PL_N * BY * BX;
    }
};

// One DUGKS step of one tile (stages 0-3).  The caller has made the tile's
// inputs visible (staged == true: in the staging area) and synchronised the
// CTA; `hook` runs right after the last read of the staged inputs.
template <int MODEL, bool WALLS, typename R, typename Hook>
__device__ __forceinline__ void tile_step(const PR<R> &P, const SR<R> &S, int first, int gin, int gout,
                                          uint32_t step, const TileCell<WALLS> &g, const Views<R> &sv,
                                          bool staged, Hook &&hook) {
    using T = typename Pair<R>::T;
    const auto sB = sv.sB;
    const auto sFS = sv.sFS;
    const auto sA = sv.sA;
    const auto sphi = sv.sphi;
    const R *stg = sv.stg, *stg_ring = sv.stg_ring;
    const int e = threadIdx.x, r = threadIdx.y;
    const int tid = r * BX + e;
    const int nx = P.nx, ny = P.ny, pitch = P.pitch;
    const int x0 = g.x0, y0 = g.y0, w = g.w, hh = g.hh, gi = g.gi, gj = g.gj;
    const bool act = g.act, ghost = g.ghost, real = g.real;
    const size_t c = g.c;

    // ---- stage 0: own deviations (f, g pairs), phi pairs of the halo-2 region
    T Pq[9];
    R sfz = R(0.);
    if (real) {
        auto plane = [&](int k) -> R { return staged ? stg[(k * BY + r) * BX + e] : S.df[(size_t)k * S.qs + c]; };
        Pq[0] = mk2(plane(PL_F), R(0.));
#pragma unroll
        for (int q = 1; q < 9; ++q) Pq[q] = mk2(plane(PL_F + q), plane(PL_G + q - 1));
        // (sum f, sum g); the Allen-Cahn pressure omits f_0
        const T za[9] = {mk2(MODEL == AC ? R(0.) : Pq[0].x, R(0.)), Pq[1], Pq[2], Pq[3], Pq[4],
                         Pq[5], Pq[6], Pq[7], Pq[8]};
        const T z = dev_sum9(za);
        sfz = z.x;
        Pq[0].y = -z.y;  // g_0 = -sum_{q>0} g_q
        sphi[r + 1][e + 1] = mk2(plane(PL_PHI), plane(PL_PHI + 1));
    } else if (act && WALLS) {
        // ghost phi: the previous step's extrapolation (Ark/Cpp/Boundary.cpp:38-63)
        const size_t gr = gphi_row(gin, gj < 0 ? 0 : 1);
        sphi[r + 1][e + 1] = mk2(S.gphi[gr * pitch + gi], S.gphi[(gr + 1) * pitch + gi]);
    }
    {   // ring of the phi region
        const int nr = g.nring();
        for (int k = tid; k < nr; k += BX * BY) {
            int re, rr;
            g.ring(k, re, rr);
            const int ri = wrapi(x0 + re - 1, nx);
            int rj = y0 + rr - 1;
            T v = mk2(R(0.), R(0.));
            if (WALLS && (rj < -1 || rj > ny)) {
                v = mk2(R(0.), R(0.));  // never read: no real cell of this tile reaches it
            } else if (WALLS && (rj == -1 || rj == ny)) {
                const size_t gr = gphi_row(gin, rj < 0 ? 0 : 1);
                v = mk2(S.gphi[gr * pitch + ri], S.gphi[(gr + 1) * pitch + ri]);
            } else {
                if (!WALLS) rj = wrapi(rj, ny);
                const size_t cc = (size_t)rj * pitch + ri;
                v = staged ? mk2(stg_ring[k], stg_ring[RING_MAX + k]) : mk2(S.phi[cc], S.phi[S.qs + cc]);
            }
            sphi[rr + 1][re + 1] = v;
        }
    }
    __syncthreads();

    // ---- stage 1: macros, MacroSource, f-bar-plus of every real cell of the region
    R phi = R(0.), U = R(0.), V = R(0.);
    T inc[9];  // collision increments B - T of this cell
    R src[6];
    if (real) {
        R a6[A_N];
        if (MODEL != AC && !first) {
#pragma unroll
            for (int k = 0; k < A_N; ++k)
                a6[k] = staged ? stg[((PL_AUX + k) * BY + r) * BX + e] : S.aux[(size_t)k * S.qs + c];
        }
        // sphi[r+1][e+1] is this cell
        const T ph[8] = {sphi[r + 1][e + 2], sphi[r + 1][e], sphi[r + 2][e + 1], sphi[r][e + 1],
                         sphi[r + 2][e + 2], sphi[r + 2][e], sphi[r][e + 2], sphi[r][e]};
        collide_cell<MODEL, R>(P, S, c, first, Pq, sfz, a6, sphi[r + 1][e + 1], ph, inc, src, phi, U, V);
#pragma unroll
        for (int q = 0; q < 9; ++q) sB[q][r][e] = add2(Pq[q], inc[q]);
#pragma unroll
        for (int k = 0; k < 6; ++k) sA[k][r][e] = src[k];
    }
    if (WALLS) {
        __syncthreads();
        // P2: ghost rows of f-bar-plus and of the averaged fields (2 a0 - a1)
        if (act && ghost) {
            const int r0 = gj < 0 ? r + 1 : r - 1, r1 = gj < 0 ? r + 2 : r - 2;
            const T two = mk2(R(2.), R(2.));
#pragma unroll
            for (int q = 0; q < 9; ++q) sB[q][r][e] = sub2(mul2(two, sB[q][r0][e]), sB[q][r1][e]);
#pragma unroll
            for (int k = 0; k < 6; ++k) sA[k][r][e] = R(2.) * sA[k][r0][e] - sA[k][r1][e];
        }
        // ghost phi for the next step's MacroSource, written by the tile owning the row
        if (real && e >= 1 && e <= w && r >= 1 && r <= hh) {
            if (gj == 0 || gj == ny - 1) {
                const int side = gj == 0 ? 0 : 1;
                const T gv = ghost_pair(sphi[r + 1][e + 1], side == 0 ? sphi[r + 2][e + 1] : sphi[r][e + 1]);
                const size_t gr = gphi_row(gout, side);
                S.gphi[gr * pitch + gi] = gv.x;
                S.gphi[(gr + 1) * pitch + gi] = gv.y;
            }
        }
    }
    __syncthreads();
    hook();  // every read of the staged inputs of this tile is done

    // phi pair of the region cell (rr, ee) as the faces and the update see it: at a
    // wall the ghost row of f-bar-plus is 2 B_0 - B_1 of this step, so its phi is
    // 2 phi_0 - phi_1 of this step (not the previous step's ghost MacroSource reads)
    auto phiB = [&](int rr, int ee) -> T {
        if (WALLS) {
            const int jj = y0 + rr - 1;
            if (jj == -1) return ghost_pair(sphi[rr + 2][ee + 1], sphi[rr + 3][ee + 1]);
            if (jj == ny) return ghost_pair(sphi[rr][ee + 1], sphi[rr - 1][ee + 1]);
        }
        return sphi[rr + 1][ee + 1];
    };
    // ---- stage 2: west x-face and south y-face of this thread's cell
    T FW[6], FSo[6];
    const bool do_x = act && e >= 1 && r >= 1 && r <= hh;           // faces x0-1|x0 .. x0+w-1|x0+w
    const bool do_y = act && r >= 1 && e >= 1 && e <= w;            // faces below rows 0..hh (hh+1 with the top)
    if (do_x) {
        R av[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) av[k] = R(0.5) * (sA[k][r][e - 1] + sA[k][r][e]);
        const FacePhi<R> fp =
            face_phi_x(phiB(r, e - 1), phiB(r, e), phiB(r + 1, e), phiB(r - 1, e), phiB(r + 1, e - 1), phiB(r - 1, e - 1));
        face_flux<MODEL, true, R>(
            P, [&](int q) { return sB[q][r][e - 1]; }, [&](int q) { return sB[q][r][e]; },
            [&](int q) {
                return add2(sub2(sB[q][r + 1][e], sB[q][r - 1][e]), sub2(sB[q][r + 1][e - 1], sB[q][r - 1][e - 1]));
            },
            av, fp, 0, FW);
    }
    if (do_y) {
        R av[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) av[k] = R(0.5) * (sA[k][r - 1][e] + sA[k][r][e]);
        const int wall = (WALLS && gj == 0) ? 1 : ((WALLS && gj == ny) ? 2 : 0);
        const FacePhi<R> fp =
            face_phi_y(phiB(r - 1, e), phiB(r, e), phiB(r, e - 1), phiB(r, e + 1), phiB(r - 1, e - 1), phiB(r - 1, e + 1));
        face_flux<MODEL, false, R>(
            P, [&](int q) { return sB[q][r - 1][e]; }, [&](int q) { return sB[q][r][e]; },
            [&](int q) {
                return add2(sub2(sB[q][r][e - 1], sB[q][r][e + 1]), sub2(sB[q][r - 1][e - 1], sB[q][r - 1][e + 1]));
            },
            av, fp, wall, FSo);
    }
    if (do_y) {
#pragma unroll
        for (int s = 0; s < 6; ++s) sFS[s][r][e] = FSo[s];
    }
    // east face = west face of the next lane
    T FE[6];
#pragma unroll
    for (int s = 0; s < 6; ++s) {
        const T v = do_x ? FW[s] : mk2(R(0.), R(0.));
        FE[s] = mk2(__shfl_down_sync(0xffffffffu, v.x, 1), __shfl_down_sync(0xffffffffu, v.y, 1));
    }
    __syncthreads();

    // ---- stage 3: finite-volume update of the interior cells (Update_phi_T) + aux
    if (real && e >= 1 && e <= w && r >= 1 && r <= hh) {
        T FN[6], dn[9];
#pragma unroll
        for (int s = 0; s < 6; ++s) FN[s] = sFS[s][r + 1][e];
        const R half_dtv = R(0.5) * P.dtV;
        const R px = half_dtv * pdiff(phiB(r, e - 1), phiB(r, e + 1));
        const R py = half_dtv * pdiff(phiB(r - 1, e), phiB(r + 1, e));
        R dphi;
        update_cell<R>(P, Pq, inc, FW, FE, FSo, FN, px, py, dn, dphi);
        S.odf[c] = dn[0].x;
#pragma unroll
        for (int q = 1; q < 9; ++q) {
            S.odf[(size_t)q * S.qs + c] = dn[q].x;
            S.odg[(size_t)(q - 1) * S.qs + c] = dn[q].y;
        }
        const T pn = phi_add(sphi[r + 1][e + 1], dphi);
        S.ophi[c] = pn.x;
        S.ophi[S.qs + c] = pn.y;
        if (MODEL != AC) {  // AC: u = 0, the next step needs no previous force, gradient or phi*u
            S.oaux[A_FX * S.qs + c] = src[4];
            S.oaux[A_FY * S.qs + c] = src[5];
            S.oaux[A_RHOX * S.qs + c] = src[2];
            S.oaux[A_RHOY * S.qs + c] = src[3];
            S.oaux[A_PPU * S.qs + c] = phi * U;
            S.oaux[A_PPV * S.qs + c] = phi * V;
        }
    }
}

// Persistent kernel: each CTA (one per SM) walks the tiles t = blockIdx.x,
// blockIdx.x + gridDim.x, ...; tile t + gridDim.x's inputs are in flight while
// tile t computes.
template <int MODEL, bool WALLS, typename R>
__global__ void __launch_bounds__(BX *BY, 1) k_step32(PR<R> P, SR<R> S, int first, int gin, int gout,
                                                      uint32_t step, int ntx, int ntiles) {
    constexpr bool PF = prefetched<R>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Views<R> sv(smem_raw);
    const int e = threadIdx.x, r = threadIdx.y, tid = r * BX + e;
    if constexpr (PF) {
        if ((int)blockIdx.x < ntiles)
            prefetch_tile<MODEL, WALLS>(P, S, blockIdx.x, ntx, e, r, tid, sv.stg, sv.stg_ring);
    }
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const TileCell<WALLS> g(t, ntx, e, r, P.nx, P.ny, P.pitch);
        if constexpr (PF) cp_async_wait_all();
        __syncthreads();  // staged inputs visible; the previous tile is done with shared memory
        tile_step<MODEL, WALLS, R>(P, S, first, gin, gout, step, g, sv, PF, [&] {
            if constexpr (PF) {
                if (t + (int)gridDim.x < ntiles)
                    prefetch_tile<MODEL, WALLS>(P, S, t + gridDim.x, ntx, e, r, tid, sv.stg, sv.stg_ring);
            }
        });
    }
}

// ---- many cases in one launch (serving): a case table in constant memory and
// a tile table (case slot, tile of that case) in device memory.  Each tile
// runs the same tile_step as the single-case kernel with its own case's
// constants, state and step number, so a case's result does not depend on
// what else is in the launch.
struct BatchCase {
    P32 P;
    S32 S[2];  // state views for even / odd step numbers (ping-pong buffers)
    int ntx;   // tiles per row
    int pad;
};
__constant__ BatchCase c_batch[BATCH_MAX_CASES];

// tiles[t] = (case slot, tile index within the case), all cases of one model
// and wall kind; case_base[slot] = the case's step number at the start of this
// launch sequence, kstep = the launch within the sequence; tiles of a case
// whose step number reached case_stop are skipped.
template <int MODEL, bool WALLS>
__global__ void __launch_bounds__(BX *BY, 1) k_batch32(const int2 *__restrict__ tiles, int ntiles, int kstep,
                                                       const int *__restrict__ case_base,
                                                       const int *__restrict__ case_stop) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Views<float> sv(smem_raw);
    const int e = threadIdx.x, r = threadIdx.y, tid = r * BX + e;
    auto issue = [&](int t) {
        if (t >= ntiles) return;
        const int2 bt = tiles[t];
        const int sn = case_base[bt.x] + kstep;
        if (sn >= case_stop[bt.x]) return;
        const BatchCase &B = c_batch[bt.x];
        prefetch_tile<MODEL, WALLS>(B.P, B.S[sn & 1], bt.y, B.ntx, e, r, tid, sv.stg, sv.stg_ring);
    };
    issue(blockIdx.x);
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int2 bt = tiles[t];
        const int sn = case_base[bt.x] + kstep;
        if (sn >= case_stop[bt.x]) {  // the whole CTA skips: nothing staged for this tile
            issue(t + gridDim.x);
            continue;
        }
        const BatchCase &B = c_batch[bt.x];
        const int par = sn & 1;
        cp_async_wait_all();
        __syncthreads();
        const TileCell<WALLS> g(bt.y, B.ntx, e, r, B.P.nx, B.P.ny, B.P.pitch);
        tile_step<MODEL, WALLS, float>(B.P, B.S[par], sn == 0, par, par ^ 1, (uint32_t)sn, g, sv, true,
                                       [&] { issue(t + gridDim.x); });
    }
}

// The same in the streaming form: items (case slot, strip, first row, end row) of the
// cases of one model and wall kind, each run by one warp with stream_item and its
// case's constants, state and step number (per-lane row loads: no tensor map per case).
// Items of a case whose step number reached case_stop are skipped.
template <int MODEL, bool WALLS>
__global__ void __launch_bounds__(WPB * 32, STREAM_MIN_BLOCKS) k_streamb32(const int4 *__restrict__ items, int nitems, int kstep,
                                                        const int *__restrict__ case_base,
                                                        const int *__restrict__ case_stop) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float *wbase = reinterpret_cast<float *>(smem_raw) + (size_t)wib * WARP_F;
    float *stg = wbase, *bring = wbase + STG_F, *aring = wbase + STG_F + BR_F;
    uint32_t phases = 0;
    const int gw = blockIdx.x * WPB + wib, nw = gridDim.x * WPB;
    for (int it = gw; it < nitems; it += nw) {
        const int4 t = items[it];
        const int sn = case_base[t.x] + kstep;
        if (sn >= case_stop[t.x]) continue;
        const BatchCase &B = c_batch[t.x];
        const int par = sn & 1;
        stream_item<MODEL, WALLS, false>(B.P, B.S[par], sn == 0, par, par ^ 1, (uint32_t)sn, t.y, t.z, t.w, false,
                                         nullptr, 0, nullptr, stg, bring, aring, 0u, phases, lane);
    }
}

// case_base[slots[k]] += n for the k < count slots of a launch sequence
__global__ void k_batch_advance(int *case_base, const int *slots, int count, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < count) case_base[slots[k]] += n;
}

// S: the case's state views for its next step, number `step`
cudaError_t batch_set_case(int slot, const P32 &P, const S32 &S, int64_t step, cudaStream_t st) {
    if (slot < 0 || slot >= BATCH_MAX_CASES) return cudaErrorInvalidValue;
    BatchCase b{};
    b.P = P;
    b.S[step & 1] = S;
    b.S[(step & 1) ^ 1] = S;
    swap_io(b.S[(step & 1) ^ 1]);
    b.ntx = (P.nx + TW - 1) / TW;
    return cudaMemcpyToSymbolAsync(c_batch, &b, sizeof(b), (size_t)slot * sizeof(BatchCase), cudaMemcpyHostToDevice,
                                   st);
}

int batch_tiles_of(int nx, int ny) { return ((nx + TW - 1) / TW) * ((ny + TH - 1) / TH); }

static int g_batch_nsm = 0;  // SMs of the device, set by batch_prepare

template <int MODEL, bool WALLS>
static cudaError_t batch_attr() {
    return cudaFuncSetAttribute(k_batch32<MODEL, WALLS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(smem_elems<float>() * sizeof(float)));
}

static int g_streamb_blocks = 0;  // resident blocks of k_streamb32 per SM, set by batch_prepare

template <int MODEL, bool WALLS>
static cudaError_t streamb_attr() {
    cudaError_t e = cudaFuncSetAttribute(k_streamb32<MODEL, WALLS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)STREAM_SMEM);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_streamb32<MODEL, WALLS>, WPB * 32, STREAM_SMEM);
    if (e != cudaSuccess) return e;
    if (per_sm <= 0) return cudaErrorInvalidConfiguration;
    g_streamb_blocks = g_streamb_blocks ? std::min(g_streamb_blocks, per_sm) : per_sm;
    return cudaSuccess;
}

// kernel attributes of the batched launches; called before any stream capture
cudaError_t batch_prepare() {
    cudaError_t e;
    if ((e = batch_attr<AC, false>()) != cudaSuccess) return e;
    if ((e = batch_attr<AC, true>()) != cudaSuccess) return e;
    if ((e = batch_attr<HCZ, false>()) != cudaSuccess) return e;
    if ((e = batch_attr<HCZ, true>()) != cudaSuccess) return e;
    if ((e = streamb_attr<AC, false>()) != cudaSuccess) return e;
    if ((e = streamb_attr<AC, true>()) != cudaSuccess) return e;
    if ((e = streamb_attr<HCZ, false>()) != cudaSuccess) return e;
    if ((e = streamb_attr<HCZ, true>()) != cudaSuccess) return e;
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    return cudaDeviceGetAttribute(&g_batch_nsm, cudaDevAttrMultiProcessorCount, dev);
}

template <int MODEL, bool WALLS>
static cudaError_t launch_batch_t(const int2 *tiles, int ntiles, int kstep, const int *case_base,
                                  const int *case_stop, cudaStream_t st) {
    if (g_batch_nsm <= 0) return cudaErrorNotReady;
    const size_t bytes = smem_elems<float>() * sizeof(float);
    k_batch32<MODEL, WALLS><<<min(ntiles, g_batch_nsm), dim3(BX, BY), bytes, st>>>(tiles, ntiles, kstep,
                                                                                    case_base, case_stop);
    return cudaGetLastError();
}

cudaError_t launch_batch32(int model, int walls, const int2 *tiles, int ntiles, int kstep, const int *case_base,
                           const int *case_stop, cudaStream_t st, int64_t *launches) {
    if (ntiles <= 0) return cudaSuccess;
    cudaError_t e = cudaErrorInvalidValue;
    switch (model * 2 + (walls ? 1 : 0)) {
        case AC * 2 + 0: e = launch_batch_t<AC, false>(tiles, ntiles, kstep, case_base, case_stop, st); break;
        case AC * 2 + 1: e = launch_batch_t<AC, true>(tiles, ntiles, kstep, case_base, case_stop, st); break;
        case HCZ * 2 + 0: e = launch_batch_t<HCZ, false>(tiles, ntiles, kstep, case_base, case_stop, st); break;
        case HCZ * 2 + 1: e = launch_batch_t<HCZ, true>(tiles, ntiles, kstep, case_base, case_stop, st); break;
        default: break;
    }
    if (e == cudaSuccess) *launches += 1;
    return e;
}

// Items of one k_streamb32 launch over the cases (slot, nx, ny), each with ny >= 8:
// every case in strips of SW columns and row segments of one common length, chosen
// like the single-case step's (stream_segment_rows): the fill of the last round of
// items over the resident warps times the share of the rows that are not warm-up.
void stream_batch_items(const std::vector<int3> &cases, std::vector<int4> &items) {
    items.clear();
    if (cases.empty()) return;
    const double warps = (double)std::max(1, g_batch_nsm * g_streamb_blocks * WPB);
    int maxny = 0;
    for (const int3 &c : cases) maxny = std::max(maxny, c.z);
    int best = std::min(32, maxny);
    double best_eff = -1.0;
    for (int len = std::min(16, maxny); len <= maxny; ++len) {
        double n = 0.0, rows = 0.0, warm = 0.0;
        for (const int3 &c : cases) {
            const int strips = (c.y + SW - 1) / SW, segs = (c.z + len - 1) / len;
            n += (double)strips * segs;
            rows += (double)strips * c.z;
            warm += 4.0 * strips * segs;
        }
        const double waves = n / warps;
        const double eff = waves / std::ceil(waves) * (rows / (rows + warm));
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = len;
        }
    }
    for (const int3 &c : cases) {
        const int strips = (c.y + SW - 1) / SW;
        for (int y0 = 0; y0 < c.z; y0 += best)
            for (int st = 0; st < strips; ++st) items.push_back(make_int4(c.x, st, y0, std::min(y0 + best, c.z)));
    }
}

template <int MODEL, bool WALLS>
static cudaError_t launch_streamb_t(const int4 *items, int nitems, int kstep, const int *case_base,
                                    const int *case_stop, cudaStream_t st) {
    if (g_batch_nsm <= 0 || g_streamb_blocks <= 0) return cudaErrorNotReady;
    const int blocks = std::min((nitems + WPB - 1) / WPB, g_batch_nsm * g_streamb_blocks);
    k_streamb32<MODEL, WALLS><<<blocks, WPB * 32, STREAM_SMEM, st>>>(items, nitems, kstep, case_base, case_stop);
    return cudaGetLastError();
}

cudaError_t launch_streamb32(int model, int walls, const int4 *items, int nitems, int kstep, const int *case_base,
                             const int *case_stop, cudaStream_t st, int64_t *launches) {
    if (nitems <= 0) return cudaSuccess;
    cudaError_t e = cudaErrorInvalidValue;
    switch (model * 2 + (walls ? 1 : 0)) {
        case AC * 2 + 0: e = launch_streamb_t<AC, false>(items, nitems, kstep, case_base, case_stop, st); break;
        case AC * 2 + 1: e = launch_streamb_t<AC, true>(items, nitems, kstep, case_base, case_stop, st); break;
        case HCZ * 2 + 0: e = launch_streamb_t<HCZ, false>(items, nitems, kstep, case_base, case_stop, st); break;
        case HCZ * 2 + 1: e = launch_streamb_t<HCZ, true>(items, nitems, kstep, case_base, case_stop, st); break;
        default: break;
    }
    if (e == cudaSuccess) *launches += 1;
    return e;
}

cudaError_t launch_batch_advance(int *case_base, const int *slots, int count, int n, cudaStream_t st,
                                 int64_t *launches) {
    if (count <= 0) return cudaSuccess;
    k_batch_advance<<<(count + 127) / 128, 128, 0, st>>>(case_base, slots, count, n);
    *launches += 1;
    return cudaGetLastError();
}

// Macroscopic fields of the FP32 state as FP64 arrays: the quantities the
// reference holds after Update_MacroVar + MacroSource of the last step.
template <int MODEL, bool WALLS, typename R>
__global__ void __launch_bounds__(256) k_macros32(PR<R> P, SR<R> S, double *rho_o, double *u_o, double *v_o,
                                                  double *p_o, double *phi_o, int opitch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= P.nx || j >= P.ny) return;
    const size_t c = (size_t)j * P.pitch + i;
    R df[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) df[q] = S.df[(size_t)q * S.qs + c];
    const double phid = (double)S.phi[c] + (double)S.phi[S.qs + c];
    const R phi = (R)phid;
    R rho, U, V, dp;
    if (MODEL == AC)
        cell_macros<MODEL, R>(P, df, phi, R(0), R(0), R(0), R(0), rho, U, V, dp);
    else
        cell_macros<MODEL, R>(P, df, phi, S.aux[A_FX * S.qs + c], S.aux[A_FY * S.qs + c], S.aux[A_RHOX * S.qs + c],
                              S.aux[A_RHOY * S.qs + c], rho, U, V, dp);
    const size_t o = (size_t)j * opitch + i;
    rho_o[o] = (double)P.aPhi * phid + (double)P.bPhi;
    u_o[o] = U;
    v_o[o] = V;
    p_o[o] = (double)P.p0 + (double)dp;
    phi_o[o] = phid;
}

// One FP64 plane (dense [ny][nx], as the C ABI passes it) to the storage type,
// minus a rest value: dst[j][i] = (R)(src[j][i] - sub)
template <typename R>
__global__ void __launch_bounds__(256) k_plane_from_f64(R *dst, int dpitch, const double *__restrict__ src, int nx,
                                                        int ny, double sub) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= nx || j >= ny) return;
    dst[(size_t)j * dpitch + i] = (R)(src[(size_t)j * nx + i] - sub);
}

template <typename R>
cudaError_t launch_plane_from_f64(R *dst, int dpitch, const double *src, int nx, int ny, double sub,
                                  cudaStream_t st, int64_t *launches) {
    const dim3 grd((nx + 255) / 256, ny);
    k_plane_from_f64<R><<<grd, 256, 0, st>>>(dst, dpitch, src, nx, ny, sub);
    *launches += 1;
    return cudaGetLastError();
}
template cudaError_t launch_plane_from_f64<float>(float *, int, const double *, int, int, double, cudaStream_t,
                                                  int64_t *);
template cudaError_t launch_plane_from_f64<double>(double *, int, const double *, int, int, double, cudaStream_t,
                                                   int64_t *);

// The phase field of an FP64 state h [9][ny][nx] (dense, as the C ABI passes it) in
// the storage layout: phi = sum_q h_q as a pair (head, tail) and g_q = h_q - w_q phi
// for q = 1..8, one plane every qs elements from g and phi.
template <typename R>
__global__ void __launch_bounds__(256) k_phase_from_f64(R *g, R *phi, size_t qs, int pitch,
                                                        const double *__restrict__ h, int nx, int ny) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= nx || j >= ny) return;
    const size_t n = (size_t)nx * ny, sidx = (size_t)j * nx + i, d = (size_t)j * pitch + i;
    double hq[9], ph = 0.0;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        hq[q] = h[q * n + sidx];
        ph += hq[q];
    }
    const R hi = (R)ph;
    phi[d] = hi;
    phi[qs + d] = (R)(ph - (double)hi);
    // separately rounded product and difference (no contraction): the same doubles as
    // the host-side split of a slab partition's initial state
#pragma unroll
    for (int q = 1; q < 9; ++q) g[(size_t)(q - 1) * qs + d] = (R)__dsub_rn(hq[q], __dmul_rn(d2q9_w(q), ph));
}

template <typename R>
cudaError_t launch_phase_from_f64(R *g, R *phi, size_t qs, int pitch, const double *h, int nx, int ny,
                                  cudaStream_t st, int64_t *launches) {
    const dim3 grd((nx + 255) / 256, ny);
    k_phase_from_f64<R><<<grd, 256, 0, st>>>(g, phi, qs, pitch, h, nx, ny);
    *launches += 1;
    return cudaGetLastError();
}
template cudaError_t launch_phase_from_f64<float>(float *, float *, size_t, int, const double *, int, int,
                                                  cudaStream_t, int64_t *);
template cudaError_t launch_phase_from_f64<double>(double *, double *, size_t, int, const double *, int, int,
                                                   cudaStream_t, int64_t *);

// tau, Fx, Fy of a deviation-storage case in FP64, for output: tau is Tau0
// after the first step (before it, the initialisation's, in the init planes);
// F = mu grad(phi) (+ gravity) with the MacroSource stencil
// (Ark/Cpp/SourceM.cpp:35-62) on the FP64 phi field, wall ghost rows
// extrapolated as 2 phi_0 - phi_1 (Ark/Cpp/Boundary.cpp:38-63).
template <typename R>
__global__ void __launch_bounds__(256) k_out_forces(PR<R> P, const double *__restrict__ phi,
                                                    const double *__restrict__ rho, int opitch,
                                                    const R *__restrict__ init_tau, int first, double *tau,
                                                    double *fx, double *fy) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= P.nx || j >= P.ny) return;
    auto at = [&](int ii, int jj) -> double {
        ii = wrapi(ii, P.nx);
        if (P.walls) {
            if (jj < 0) return 2.0 * phi[(size_t)ii] - phi[(size_t)opitch + ii];
            if (jj >= P.ny)
                return 2.0 * phi[(size_t)(P.ny - 1) * opitch + ii] - phi[(size_t)(P.ny - 2) * opitch + ii];
        } else {
            jj = wrapi(jj, P.ny);
        }
        return phi[(size_t)jj * opitch + ii];
    };
    const double c = at(i, j), E = at(i + 1, j), W = at(i - 1, j), N = at(i, j + 1), S = at(i, j - 1);
    const double NE = at(i + 1, j + 1), NW = at(i - 1, j + 1), SE = at(i + 1, j - 1), SW = at(i - 1, j - 1);
    double gx = (4.0 * (E - W) + ((NE - NW) + (SE - SW))) * (double)P.inv_12dx;
    double gy = (4.0 * (N - S) + ((NE - SE) + (NW - SW))) * (double)P.inv_12dy;
    const double lap = (4.0 * ((E + W) + (N + S)) + ((NE + SW) + (NW + SE)) - 20.0 * c) * (double)P.inv_6dd;
    if (fabs(gx) < DUGKS_F32_GCLAMP) gx = 0.0;
    if (fabs(gy) < DUGKS_F32_GCLAMP) gy = 0.0;
    const double PhiL = P.PhiL, PhiV = P.PhiV;
    const double F = 2.0 * (double)P.Beta * (c - PhiL) * (c - PhiV) * (2.0 * c - PhiL - PhiV) - (double)P.Kappa * lap;
    const size_t o = (size_t)j * opitch + i;
    fx[o] = F * gx;
    fy[o] = F * gy - (P.gravity ? (double)P.Gy * (rho[o] - (double)P.RhoL) : 0.0);
    tau[o] = first ? (double)init_tau[(size_t)j * P.pitch + i] : (double)P.tauf;
}

template <typename R>
void launch_out_forces(const PR<R> &P, const SR<R> &S, const double *phi, const double *rho, int opitch, int first,
                       double *tau, double *fx, double *fy, cudaStream_t st, int64_t *launches) {
    const dim3 blk(32, 8);
    const dim3 grd((P.nx + 31) / 32, (P.ny + 7) / 8);
    k_out_forces<R><<<grd, blk, 0, st>>>(P, phi, rho, opitch, S.init + (size_t)I_TAU * S.qs, first, tau, fx, fy);
    *launches += 1;
}
template void launch_out_forces<float>(const PR<float> &, const SR<float> &, const double *, const double *, int, int,
                                       double *, double *, double *, cudaStream_t, int64_t *);
template void launch_out_forces<double>(const PR<double> &, const SR<double> &, const double *, const double *, int,
                                        int, double *, double *, double *, cudaStream_t, int64_t *);

template <int MODEL, bool WALLS, typename R>
static cudaError_t launch_t(const PR<R> &P, const SR<R> &S, int first, int gin, int gout, cudaStream_t st,
                            uint32_t step) {
    const size_t bytes = smem_elems<R>() * sizeof(R);
    static bool attr_set = false;  // per instantiation; idempotent, set before the first launch
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_step32<MODEL, WALLS, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)bytes);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    static int nsm = 0;  // SMs of the device (one persistent CTA each)
    if (!nsm) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
    }
    const int ntx = (P.nx + TW - 1) / TW, nty = (P.ny + TH - 1) / TH, ntiles = ntx * nty;
    const dim3 blk(BX, BY);
    k_step32<MODEL, WALLS, R><<<min(ntiles, nsm), blk, bytes, st>>>(P, S, first, gin, gout, step, ntx, ntiles);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_stepR(const PR<R> &P, const SR<R> &S, int first, int gin, int gout, cudaStream_t st,
                         int64_t *launches, uint32_t step) {
    cudaError_t e = cudaErrorInvalidValue;
    switch (P.model * 2 + (P.walls ? 1 : 0)) {
        case AC * 2 + 0: e = launch_t<AC, false, R>(P, S, first, gin, gout, st, step); break;
        case AC * 2 + 1: e = launch_t<AC, true, R>(P, S, first, gin, gout, st, step); break;
        case HCZ * 2 + 0: e = launch_t<HCZ, false, R>(P, S, first, gin, gout, st, step); break;
        case HCZ * 2 + 1: e = launch_t<HCZ, true, R>(P, S, first, gin, gout, st, step); break;
        default: break;
    }
    if (e == cudaSuccess) *launches += 1;
    return e;
}

template <typename R>
void launch_macrosR(const PR<R> &P, const SR<R> &S, double *rho, double *u, double *v, double *p, double *phi,
                    int opitch, cudaStream_t st, int64_t *launches) {
    const dim3 blk(32, 8);
    const dim3 grd((P.nx + 31) / 32, (P.ny + 7) / 8);
    switch (P.model * 2 + (P.walls ? 1 : 0)) {
        case AC * 2 + 0: k_macros32<AC, false, R><<<grd, blk, 0, st>>>(P, S, rho, u, v, p, phi, opitch); break;
        case AC * 2 + 1: k_macros32<AC, true, R><<<grd, blk, 0, st>>>(P, S, rho, u, v, p, phi, opitch); break;
        case HCZ * 2 + 0: k_macros32<HCZ, false, R><<<grd, blk, 0, st>>>(P, S, rho, u, v, p, phi, opitch); break;
        case HCZ * 2 + 1: k_macros32<HCZ, true, R><<<grd, blk, 0, st>>>(P, S, rho, u, v, p, phi, opitch); break;
        default: return;
    }
    *launches += 1;
}

cudaError_t launch_step32(const P32 &P, const S32 &S, int first, int gin, int gout, cudaStream_t st,
                          int64_t *launches, uint32_t step) {
    return launch_stepR<float>(P, S, first, gin, gout, st, launches, step);
}
cudaError_t launch_step64f(const PR<double> &P, const SR<double> &S, int first, int gin, int gout,
                           cudaStream_t st, int64_t *launches, uint32_t step) {
    return launch_stepR<double>(P, S, first, gin, gout, st, launches, step);
}
void launch_macros32(const P32 &P, const S32 &S, double *rho, double *u, double *v, double *p, double *phi,
                     int opitch, cudaStream_t st, int64_t *launches) {
    launch_macrosR<float>(P, S, rho, u, v, p, phi, opitch, st, launches);
}
void launch_macros64f(const PR<double> &P, const SR<double> &S, double *rho, double *u, double *v, double *p,
                      double *phi, int opitch, cudaStream_t st, int64_t *launches) {
    launch_macrosR<double>(P, S, rho, u, v, p, phi, opitch, st, launches);
}

}  // namespace f32
}  // namespace dugks
