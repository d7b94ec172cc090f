// The streaming form of the FP32 deviation-storage step: its constants, shared-memory
// ring layout and TMA helpers (used by the single-case kernel k_stream32,
// fp32_stream.cu, and the batched serving kernel k_streamb32, fp32_fused.cu), and the
// per-warp work on one (strip, row segment) item, stream_item (run by both kernels).
//
// A warp marches a strip of 28 columns (plus a two-column halo on each side, 32
// lanes) along y through a segment of rows.  No block-wide barrier: the
// y-neighbours of a row are in the warp's own rolling buffers (shared memory), the
// x-neighbours are the adjacent lanes' entries of the same buffers (or a shuffle),
// so every warp runs independently of the others and of its block.
//
// Per row k the warp does, in order:
//   the load of row k+3's deviations into the stage ring (the phase field phi and
//     the aux of a row are read directly into registers one row ahead of their use);
//   collision of row k+1 (the sums of its deviations, macros, MacroSource on the 3x3
//     phi stencil from the phi of rows k..k+2 and the adjacent lanes, f-bar-plus)
//     into the f-bar-plus ring;
//   the y-face between rows k and k+1 (its flux is row k's north face and,
//     carried to the next row, row k+1's south face);
//   the x-faces of row k (west face per lane, east face from the next lane);
//   the update of row k.
// A segment starts four rows early (phi of rows y0-2 and y0-1, collision of row
// y0-1, the face below row y0); those rows' results are not written.  Bounce-back
// walls: ghost rows -1 and ny of f-bar-plus and of the averaged fields are
// extrapolated (2 a0 - a1) into the rings and the wall faces bounce back, as in
// the tile kernel.  The per-cell arithmetic is the tile kernel's (fp32_math.cuh)
// with the same random bits, so the kernels give bit-identical results.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "dugks_device.cuh"
#include "fp32_math.cuh"
#include "fp32_state.cuh"

namespace dugks {
namespace f32 {

constexpr int SW = 28;   // interior columns of a strip
constexpr int SEG_MAX = 128;  // longest first-choice segment (rows)
constexpr int WPB = 1;   // warps per block (one warp a block: 4.6 % faster than 2 on 8192^2)
constexpr int NSTG = 4;  // stage ring: rows k .. k+3
// resident blocks per SM the streaming kernels are compiled for: 10 one-warp blocks (up to
// 204 registers a thread; the kernel takes 168 and 12 blocks fit) ran 1.9 % faster on the
// 8192^2 step than a bound of 12 warps at 168 registers
constexpr int STREAM_MIN_BLOCKS = 10;
// per-warp shared memory, in floats:
//   stage ring [NSTG][17][32]: the raw planes (9 f, then g_1 .. g_8) of rows
//     k .. k+3, 32 columns each -- the box one TMA load writes;
//   f-bar-plus ring, per row slot: [4][32] float4 holding the pairs of directions
//     (1,2), (3,4), (5,6), (7,8), then [32] float2 holding direction 0;
//   averaged-field ring, per row slot: [32] float4 (srcx, srcy, rhox, rhoy), then
//     [32] float2 (fx, fy).
// 8- and 16-byte entries make one shared-memory instruction move two or four values.
// After the warps' regions: 4 mbarriers per warp (one per stage slot).
constexpr int STG_PLANES = PL_PHI;   // the planes a row load stages: 9 f, 8 g
constexpr int STG_SLOT = STG_PLANES * 32;  // floats per stage slot
constexpr int STG_F = NSTG * STG_SLOT;
constexpr int BR_SLOT = 9 * 32 * 2;  // floats per row slot of the f-bar-plus ring
constexpr int BR_F = 3 * BR_SLOT;
constexpr int AR_SLOT = 6 * 32;      // floats per row slot of the averaged-field ring
constexpr int AR_F = 3 * AR_SLOT;
constexpr int WARP_F = STG_F + BR_F + AR_F;
constexpr size_t STREAM_SMEM = (size_t)WPB * WARP_F * sizeof(float) + (size_t)WPB * NSTG * 8;
static_assert((STG_SLOT * 4) % 128 == 0 && (WARP_F * 4) % 128 == 0, "TMA destinations are 128-byte aligned");
static_assert((BR_SLOT * 4) % 16 == 0 && (AR_SLOT * 4) % 16 == 0, "16-byte aligned ring slots");
constexpr unsigned STG_TX_BYTES = STG_SLOT * 4;   // bytes one TMA row load delivers
constexpr int TMA_WAIT_LIMIT = 1 << 22;           // try_wait polls before a staged load is given up

__device__ __forceinline__ int m3(int j) { return (j + 6) % 3; }  // j >= -6
__device__ __forceinline__ int m4(int j) { return (j + 8) & 3; }  // j >= -8
__device__ __forceinline__ int wrap_any(int j, int n) { return ((j % n) + n) % n; }

// ---- TMA row loads completed through an mbarrier (inline PTX)
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for the phase of the given parity; true when it completed
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
    for (int it = 0; it < TMA_WAIT_LIMIT; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// one box {32 columns, 1 row, STG_PLANES planes} at (x, y, z) of a 3-D tensor map into shared memory
__device__ __forceinline__ void tma_load_row(unsigned dst, const CUtensorMap *map, int x, int y, int z, unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::
            "r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

// one row slot of the f-bar-plus ring (see above); l is a lane (column of the strip)
struct BRow {
    float *base;
    __device__ __forceinline__ float4 *quad() const { return reinterpret_cast<float4 *>(base); }
    __device__ __forceinline__ float2 *rest() const { return reinterpret_cast<float2 *>(base + 4 * 32 * 4); }
    __device__ __forceinline__ float2 get(int q, int l) const {
        if (q == 0) return rest()[l];
        const float4 v = quad()[((q - 1) >> 1) * 32 + l];
        return ((q - 1) & 1) ? make_float2(v.z, v.w) : make_float2(v.x, v.y);
    }
    __device__ __forceinline__ void put(const float2 (&b)[9], int l) const {
#pragma unroll
        for (int g = 0; g < 4; ++g)
            quad()[g * 32 + l] = make_float4(b[2 * g + 1].x, b[2 * g + 1].y, b[2 * g + 2].x, b[2 * g + 2].y);
        rest()[l] = b[0];
    }
};
// one row slot of the averaged-field ring: {srcx, srcy, rhox, rhoy, fx, fy}
struct ARow {
    float *base;
    __device__ __forceinline__ float4 *quad() const { return reinterpret_cast<float4 *>(base); }
    __device__ __forceinline__ float2 *pair() const { return reinterpret_cast<float2 *>(base + 32 * 4); }
    __device__ __forceinline__ void get(float (&a)[6], int l) const {
        const float4 v = quad()[l];
        const float2 w = pair()[l];
        a[0] = v.x, a[1] = v.y, a[2] = v.z, a[3] = v.w, a[4] = w.x, a[5] = w.y;
    }
    __device__ __forceinline__ void put(const float (&a)[6], int l) const {
        quad()[l] = make_float4(a[0], a[1], a[2], a[3]);
        pair()[l] = make_float2(a[4], a[5]);
    }
};

// One (strip, rows y0 .. y1-1) item of a step of one case.  stg, bring, aring: the
// warp's shared-memory rings; bar0, phases: its stage-slot mbarriers and their phase
// parities (TMA instances).  use of TMA for the item: tma_ok and a window that does not
// wrap around x.  NEE: the wall faces by non-equilibrium extrapolation (P.nee cases) instead
// of bounce-back.  Returns false when a TMA load did not complete (the warp must end).
template <int MODEL, bool WALLS, bool TMA, bool NEE = false>
__device__ __forceinline__ bool stream_item(const P32 &P, const S32 &S, int first, int gin, int gout, uint32_t step,
                                            int strip, int y0, int y1, bool tma_ok, const CUtensorMap *tmap_p,
                                            int zin, int *err, float *stg, float *bring, float *aring,
                                            unsigned bar0, uint32_t &phases, int lane) {
    using T = float2;
    // (f_q, g_q) of a staged row; g_0 is -sum_{q>0} g_q and is filled in by the caller
    auto STG = [&](int slot, int q) -> T {
        return mk2(stg[slot * STG_SLOT + q * 32 + lane], q ? stg[slot * STG_SLOT + (8 + q) * 32 + lane] : 0.f);
    };
    const int nx = P.nx, ny = P.ny, pitch = P.pitch;
    // the strip's window is columns hs .. hs+31 (a multiple of 4: 16-byte TMA
    // coordinates); its interior columns x0 .. x0+w-1 run over 2 .. nx+1, the
    // last strip's wrapping around the periodic x boundary
    const int hs = strip * SW, x0 = hs + 2, w = min(SW, nx + 2 - x0);
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
                    tma_load_row(smem_u32(stg + m4(j) * STG_SLOT), tmap_p, hs, row_of(j), zin, bar);
                }
            } else {
                const long long c = cell(j);
                float *d = stg + m4(j) * STG_SLOT + lane;
#pragma unroll
                for (int q = 0; q < STG_PLANES; ++q) cp_async(d + q * 32, S.df + (size_t)q * S.qs + c);
            }
        }
        if (!use_tma) cp_async_commit();
    };
    // phi of row j as a pair: a stored row, the wall ghost row (the previous step's
    // extrapolation, Ark/Cpp/Boundary.cpp:38-63, read by MacroSource only), or unused
    auto load_phi = [&](int j) -> T {
        if (j <= y1 + 1 && row_ok(j)) {
            const long long c = cell(j);
            return mk2(__ldg(S.phi + c), __ldg(S.phi + S.qs + c));
        }
        if ((wlo && j == -1) || (whi && j == ny)) {
            const size_t gr = gphi_row(gin, j < 0 ? 0 : 1);
            return mk2(S.gphi[gr * pitch + gi], S.gphi[(gr + 1) * pitch + gi]);
        }
        return mk2(0.f, 0.f);
    };
    auto from_east = [](T v) {
        return mk2(__shfl_down_sync(0xffffffffu, v.x, 1), __shfl_down_sync(0xffffffffu, v.y, 1));
    };
    auto from_west = [](T v) {
        return mk2(__shfl_up_sync(0xffffffffu, v.x, 1), __shfl_up_sync(0xffffffffu, v.y, 1));
    };
    __syncwarp();  // the previous item is done with this warp's buffers
    prefetch(y0 - 2);
    // rolling per-lane state: the phi pairs of rows k-1 .. k+2 (ph_m, ph0, ph1, ph2),
    // of row k+3 (ph_n, loaded one row ahead) and of row k-1 in the west lane
    // (ph_mw); row k's collision increments and south-face flux
    T ph_m = mk2(0.f, 0.f), ph_mw = mk2(0.f, 0.f), ph0 = mk2(0.f, 0.f), ph1 = mk2(0.f, 0.f);
    T ph2 = mk2(0.f, 0.f), ph_n = load_phi(y0 - 2);
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
        // aux of row k+2 and phi of row k+3, read directly one row ahead of their use
        const bool coll = k + 1 >= y0 - 1 && row_ok(k + 1) && colL;
        float a6n[A_N];
        if (MODEL != AC && !first && k + 2 >= y0 - 1 && row_ok(k + 2) && colL) {
            const long long c2 = cell(k + 2);
#pragma unroll
            for (int a = 0; a < A_N; ++a) a6n[a] = __ldg(S.aux + (size_t)a * S.qs + c2);
        }
        ph2 = ph_n;
        ph_n = load_phi(k + 3);
        // row k+2's raw deviations (issued one row ago) have landed
        if (use_tma) {
            if (loaded(k + 2)) {
                const int s = m4(k + 2);
                const bool ok = __all_sync(0xffffffffu, mbar_wait(bar0 + 8 * s, (phases >> s) & 1u));
                if (!ok) {
                    // a warp has one row load in flight at a time (row k+3 is issued only
                    // after row k+2 has landed), so this slot's copy is the only one that
                    // can still write the warp's shared memory: wait for it once more
                    // (bounded), then end the warp
                    if (lane == 0 && err) atomicExch(err, 1);
                    mbar_wait(bar0 + 8 * s, (phases >> s) & 1u);
                    return false;
                }
                phases ^= 1u << s;
            }
        } else {
            cp_async_wait_all();
        }
        __syncwarp();  // every lane has read slot k-1 (the update of row k-1), refilled next
        prefetch(k + 3);
        // ---- collision of row k+1
        T inc_nx[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) inc_nx[q] = mk2(0.f, 0.f);
        // 3x3 phi stencil of row k+1: rows k (S), k+1, k+2 (N); lanes +-1 (E/W)
        const T E = from_east(ph1), W = from_west(ph1);
        const T NE = from_east(ph2), NW = from_west(ph2);
        const T SE = from_east(ph0), SWv = from_west(ph0);
        {
            const int j = k + 1;
            if (coll) {
                const int sl = m4(j);
                T Pq[9];
#pragma unroll
                for (int q = 0; q < 9; ++q) Pq[q] = STG(sl, q);
                // (sum f, sum g) of the row's deviations (AC: without f_0); g_0 = -sum g
                T za[9];
#pragma unroll
                for (int q = 0; q < 9; ++q) za[q] = Pq[q];
                if (MODEL == AC) za[0].x = 0.f;
                const T z = dev_sum9(za);
                Pq[0].y = -z.y;
                const T ph[8] = {E, W, ph2, ph0, NE, NW, SE, SWv};
                const long long c = cell(j);
                float src[6], phi, U, V;
                collide_cell<MODEL, float>(P, S, c, first, Pq, z.x, a6c, ph1, ph, inc_nx, src, phi, U, V);
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
                    auto put_ghost = [&](int side, T v) {
                        const size_t gr = gphi_row(gout, side);
                        S.gphi[gr * pitch + gi] = v.x;
                        S.gphi[(gr + 1) * pitch + gi] = v.y;
                    };
                    if (wlo && j == 0) put_ghost(0, ghost_pair(ph1, ph2));
                    if (whi && j == ny - 1) put_ghost(1, ghost_pair(ph1, ph0));
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
        // phi pairs of rows k-1 and k+1 as the faces and the update of row k see them: at
        // a wall the ghost row of f-bar-plus is 2 B_0 - B_1 of this step, so its phi is
        // 2 phi_0 - phi_1 of this step (not the previous step's ghost MacroSource reads)
        const bool bot = wlo && k == 0, top = whi && k == ny - 1;
        T dn_c = ph_m, dn_w = ph_mw, up_c = ph1, up_w = W, up_e = E;
        if (bot) {
            dn_c = ghost_pair(ph0, ph1);
            dn_w = ghost_pair(SWv, W);
        }
        if (top) {
            const T mE = from_east(ph_m);
            up_c = ghost_pair(ph0, ph_m);
            up_w = ghost_pair(SWv, ph_mw);
            up_e = ghost_pair(SE, mE);
        }
        // NEE wall face of row k (side 0: below, 1: above) into F: the row's collision state
        // again (the collision ran a row earlier and kept only f-bar-plus), from its staged
        // deviations, its aux and the 3x3 phi stencil around it -- the wall rows only
        auto nee_face = [&](int side, T (&F)[6]) {
            const T mE = from_east(ph_m);  // every lane (shuffle)
            if (!interior) return;
            const int sl = m4(k);
            T Pq[9], za[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) za[q] = Pq[q] = STG(sl, q);
            if (MODEL == AC) za[0].x = 0.f;
            const T z = dev_sum9(za);
            Pq[0].y = -z.y;
            const long long c = cell(k);
            float a6[A_N];
#pragma unroll
            for (int a = 0; a < A_N; ++a) a6[a] = (MODEL != AC && !first) ? __ldg(S.aux + (size_t)a * S.qs + c) : 0.f;
            const T ph[8] = {SE, SWv, ph1, ph_m, E, W, mE, ph_mw};
            T inc[9];
            float src[6], phi, U, V;
            CellEq<float> ce;
            collide_cell<MODEL, float, true>(P, S, c, first, Pq, z.x, a6, ph0, ph, inc, src, phi, U, V, &ce);
            const float avg = side ? 0.5f * (ph0.x + up_c.x) : 0.5f * (dn_c.x + ph0.x);
            nee_wall_flux<MODEL, float>(P, ce, Pq, avg, side, F);
        };
        // ---- y-face between rows k-1 and k at the bottom wall (row 0's south face)
        if (NEE && bot) {
            nee_face(0, FS);
        } else if (bot && interior) {
            float av[6], am[6], a0[6];
            Am.get(am, lane);
            A0.get(a0, lane);
#pragma unroll
            for (int a = 0; a < 6; ++a) av[a] = 0.5f * (am[a] + a0[a]);
            const FacePhi<float> fp = face_phi_y(dn_c, ph0, SWv, SE, dn_w, ghost_pair(SE, E));
            face_flux<MODEL, false, float>(
                P, [&](int q) { return Bm.get(q, lane); }, [&](int q) { return B0.get(q, lane); },
                [&](int q) {
                    return add2(sub2(B0.get(q, lane - 1), B0.get(q, lane + 1)),
                                sub2(Bm.get(q, lane - 1), Bm.get(q, lane + 1)));
                },
                av, fp, 1, FS);
        }
        // ---- y-face between rows k and k+1 (row k's north face)
        T FN[6];
#pragma unroll
        for (int s = 0; s < 6; ++s) FN[s] = mk2(0.f, 0.f);
        const bool yface = k >= y0 - 1 && ((row_ok(k) && row_ok(k + 1)) || top);
        if (NEE && top) {
            nee_face(1, FN);
        } else if (yface && interior) {
            float av[6], a0[6], ap[6];
            A0.get(a0, lane);
            Ap.get(ap, lane);
#pragma unroll
            for (int a = 0; a < 6; ++a) av[a] = 0.5f * (a0[a] + ap[a]);
            const int wall = top ? 2 : 0;
            const FacePhi<float> fp = face_phi_y(ph0, up_c, up_w, up_e, SWv, SE);
            face_flux<MODEL, false, float>(
                P, [&](int q) { return B0.get(q, lane); }, [&](int q) { return Bp.get(q, lane); },
                [&](int q) {
                    return add2(sub2(Bp.get(q, lane - 1), Bp.get(q, lane + 1)),
                                sub2(B0.get(q, lane - 1), B0.get(q, lane + 1)));
                },
                av, fp, wall, FN);
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
            const FacePhi<float> fp = face_phi_x(SWv, ph0, up_c, dn_c, up_w, dn_w);
            face_flux<MODEL, true, float>(
                P, [&](int q) { return B0.get(q, lane - 1); }, [&](int q) { return B0.get(q, lane); },
                [&](int q) {
                    return add2(sub2(Bp.get(q, lane), Bm.get(q, lane)), sub2(Bp.get(q, lane - 1), Bm.get(q, lane - 1)));
                },
                av, fp, 0, FW);
        }
        T FE[6];
        {   // the east face's flux is the next lane's west face, through row k-1's f-bar-plus
            // slot (no longer read in this row): three 16-byte stores and loads instead of
            // twelve shuffles (lane 31 reads past its slot row, in bounds, unused)
            float4 *fq = reinterpret_cast<float4 *>(Bm.base);
#pragma unroll
            for (int g = 0; g < 3; ++g)
                fq[g * 32 + lane] = make_float4(FW[2 * g].x, FW[2 * g].y, FW[2 * g + 1].x, FW[2 * g + 1].y);
            __syncwarp();
#pragma unroll
            for (int g = 0; g < 3; ++g) {
                const float4 v = fq[g * 32 + lane + 1];
                FE[2 * g] = mk2(v.x, v.y);
                FE[2 * g + 1] = mk2(v.z, v.w);
            }
        }
        // ---- update of row k
        if (upd && interior) {
            const int sl = m4(k);
            T Pq[9], dn[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) Pq[q] = STG(sl, q);
            const long long c = cell(k);
            const float half_dtv = 0.5f * P.dtV;
            const float px = half_dtv * pdiff(SWv, SE), py = half_dtv * pdiff(dn_c, up_c);
            float dphi;
            update_cell<float>(P, Pq, inc_cur, FW, FE, FS, FN, px, py, dn, dphi);
            S.odf[c] = dn[0].x;
#pragma unroll
            for (int q = 1; q < 9; ++q) {
                S.odf[(size_t)q * S.qs + c] = dn[q].x;
                S.odg[(size_t)(q - 1) * S.qs + c] = dn[q].y;
            }
            const T pn = phi_add(ph0, dphi);
            S.ophi[c] = pn.x;
            S.ophi[S.qs + c] = pn.y;
        }
        // ---- roll the per-lane state one row up
#pragma unroll
        for (int q = 0; q < 9; ++q) inc_cur[q] = inc_nx[q];
#pragma unroll
        for (int s = 0; s < 6; ++s) FS[s] = FN[s];
        ph_m = ph0;
        ph_mw = SWv;
        ph0 = ph1;
        ph1 = ph2;
        if (MODEL != AC) {
#pragma unroll
            for (int a = 0; a < A_N; ++a) a6c[a] = a6n[a];
        }
    }
    cp_async_wait_all();  // nothing in flight into this warp's buffers
    return true;
}

}  // namespace f32
}  // namespace dugks
