// FP32 deviation-storage step with the upwind (UW) flux scheme (_FLUX_SCHEME_UW_ARK),
// periodic grids of the Allen-Cahn models (AC, HCZ).
//
// The reference's UW (Ark/Cpp/DUGKS2DSolver.cpp:196-205,540-603,689-706) takes per cell
// the 6-point gradient of f-bar-plus and h-bar-plus (Grad_VS_6points,
// Ark/Lib/GradSchemeBasic.h:95-126) and at each face extrapolates the upwind cell's value
// to x_f - hDt xi (the two cells' extrapolations averaged for the velocities along the
// face).  The gradient needs f-bar-plus of a cell's eight neighbours, so this form runs
// four launches over scratch planes (UW_PLANES, one every qs floats from U):
//   collision  -> f-bar-plus pairs, collision increments, averaged-field inputs;
//   gradients  -> cell gradients of the f-bar-plus pairs and of the phase field (the
//                 6-point one, or the least-squares / 4-point ones of DUGKS_FLUX_UW_LS /
//                 DUGKS_FLUX_UW_4P);
//   faces      -> upwind reconstruction, then the same face moments, equilibria and
//                 fluxes as the central scheme (face_state_flux);
//   update     -> the same finite-volume update (update_cell).
// The per-cell and per-face arithmetic is the central-scheme step's (collide_cell,
// face_state_flux, update_cell in fp32_math.cuh); only the reconstruction differs.
// In the split storage h_q = g_q + w_q phi, so an h extrapolation is the g extrapolation
// plus w_q times the phi extrapolation; the face works relative to w_q times the face's
// phi average, as the central face does:
//   bh_q.y = g_u + d.grad g_u + w_q (phi_u - avg + d.grad phi_u),  d = x_f - hDt xi - x_u,
// with phi_u - avg = -+(phi_n - phi_o)/2 formed from the float-float pairs.
#include <cuda_runtime.h>

#include <cstdint>

#include "fp32_math.cuh"

namespace dugks {
namespace f32 {

namespace {

constexpr int UBX = 32, UBY = 8;

struct Cells {
    int i, j, im, ip, jm, jp;
    size_t c;
};

__device__ __forceinline__ bool cell_of(const P32 &P, Cells &k) {
    k.i = blockIdx.x * UBX + threadIdx.x;
    k.j = blockIdx.y * UBY + threadIdx.y;
    if (k.i >= P.nx || k.j >= P.ny) return false;
    k.im = wrapi(k.i - 1, P.nx);
    k.ip = wrapi(k.i + 1, P.nx);
    k.jm = wrapi(k.j - 1, P.ny);
    k.jp = wrapi(k.j + 1, P.ny);
    k.c = (size_t)k.j * P.pitch + k.i;
    return true;
}

__device__ __forceinline__ size_t at(const P32 &P, int j, int i) { return (size_t)j * P.pitch + i; }

__device__ __forceinline__ float2 phi_at(const S32 &S, size_t c) { return mk2(S.phi[c], S.phi[S.qs + c]); }

// the stored deviations of a cell as (f, g) pairs, g_0 = -sum g; sfz = sum f (AC: without f_0)
template <int MODEL>
__device__ __forceinline__ void load_cell(const S32 &S, size_t c, float2 (&Pq)[9], float &sfz) {
    Pq[0] = mk2(S.df[c], 0.f);
#pragma unroll
    for (int q = 1; q < 9; ++q) Pq[q] = mk2(S.df[(size_t)q * S.qs + c], S.dg[(size_t)(q - 1) * S.qs + c]);
    const float2 za[9] = {mk2(MODEL == AC ? 0.f : Pq[0].x, 0.f), Pq[1], Pq[2], Pq[3], Pq[4],
                          Pq[5], Pq[6], Pq[7], Pq[8]};
    const float2 z = dev_sum9(za);
    sfz = z.x;
    Pq[0].y = -z.y;
}

}  // namespace

// Collision of every cell: f-bar-plus pairs (B), the increments B - T (INC), the
// averaged-field inputs (A) and, HCZ, the MacroSource outputs the next step reads.
template <int MODEL>
__global__ void __launch_bounds__(UBX *UBY) k_uw32_collide(P32 P, S32 S, float *U, int first) {
    Cells k;
    if (!cell_of(P, k)) return;
    const size_t qs = S.qs, c = k.c;
    float2 Pq[9];
    float sfz;
    load_cell<MODEL>(S, c, Pq, sfz);
    float a6[A_N];
#pragma unroll
    for (int a = 0; a < A_N; ++a) a6[a] = (MODEL != AC && !first) ? S.aux[(size_t)a * qs + c] : 0.f;
    const float2 ph[8] = {phi_at(S, at(P, k.j, k.ip)),  phi_at(S, at(P, k.j, k.im)),  phi_at(S, at(P, k.jp, k.i)),
                          phi_at(S, at(P, k.jm, k.i)),  phi_at(S, at(P, k.jp, k.ip)), phi_at(S, at(P, k.jp, k.im)),
                          phi_at(S, at(P, k.jm, k.ip)), phi_at(S, at(P, k.jm, k.im))};
    float2 inc[9];
    float src[6], phi, Uu, Vv;
    collide_cell<MODEL, float>(P, S, (long long)c, first, Pq, sfz, a6, phi_at(S, c), ph, inc, src, phi, Uu, Vv);
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const float2 b = add2(Pq[q], inc[q]);
        U[(size_t)(UW_B + q) * qs + c] = b.x;
        U[(size_t)(UW_B + 9 + q) * qs + c] = b.y;
        U[(size_t)(UW_INC + q) * qs + c] = inc[q].x;
        U[(size_t)(UW_INC + 9 + q) * qs + c] = inc[q].y;
    }
#pragma unroll
    for (int a = 0; a < 6; ++a) U[(size_t)(UW_A + a) * qs + c] = src[a];
    if (MODEL != AC) {
        S.oaux[A_FX * qs + c] = src[4];
        S.oaux[A_FY * qs + c] = src[5];
        S.oaux[A_RHOX * qs + c] = src[2];
        S.oaux[A_RHOY * qs + c] = src[3];
        S.oaux[A_PPU * qs + c] = phi * Uu;
        S.oaux[A_PPV * qs + c] = phi * Vv;
    }
}

// 6-point gradients (axis neighbours 4, diagonals 1, over 12 dx) of the 18 f-bar-plus
// planes and of phi (from pair differences), or with uw_grad the least-squares and the
// 4-point gradients, which on unit cells are both (E - W) / 2 and (N - S) / 2 (their
// different FP64 roundings are below FP32's).  blockIdx.z: a third of the planes each (one
// thread over all 18 took 4x as long: its dependent neighbour loads, not the bandwidth,
// set the pace); the first third also the phase field's.
constexpr int UW_GRAD_SLICES = 3;
__global__ void __launch_bounds__(UBX *UBY) k_uw32_grad(P32 P, S32 S, float *U) {
    Cells k;
    if (!cell_of(P, k)) return;
    const size_t qs = S.qs, c = k.c;
    const size_t cE = at(P, k.j, k.ip), cW = at(P, k.j, k.im), cN = at(P, k.jp, k.i), cS = at(P, k.jm, k.i);
    const size_t cNE = at(P, k.jp, k.ip), cNW = at(P, k.jp, k.im), cSE = at(P, k.jm, k.ip), cSW = at(P, k.jm, k.im);
    auto gx = [&](float s) { return s * P.inv_12dx; };
    auto gy = [&](float s) { return s * P.inv_12dy; };
    const bool six = P.uw_grad == 0;
    constexpr int PER = 18 / UW_GRAD_SLICES;
#pragma unroll
    for (int p = blockIdx.z * PER; p < (int)(blockIdx.z + 1) * PER; ++p) {
        const float *B = U + (size_t)(UW_B + p) * qs;
        const float E = B[cE], W = B[cW], N = B[cN], Sv = B[cS];
        float x, y;
        if (six) {
            const float NE = B[cNE], NW = B[cNW], SE = B[cSE], SW = B[cSW];
            x = gx(fmaf(4.f, E - W, (NE - NW) + (SE - SW)));
            y = gy(fmaf(4.f, N - Sv, (NE - SE) + (NW - SW)));
        } else {
            x = 0.5f * (E - W);
            y = 0.5f * (N - Sv);
        }
        U[(size_t)(UW_GX + p) * qs + c] = x;
        U[(size_t)(UW_GY + p) * qs + c] = y;
    }
    if (blockIdx.z != 0) return;
    const float2 E = phi_at(S, cE), W = phi_at(S, cW), N = phi_at(S, cN), Sv = phi_at(S, cS);
    float x, y;
    if (six) {
        const float2 NE = phi_at(S, cNE), NW = phi_at(S, cNW), SE = phi_at(S, cSE), SW = phi_at(S, cSW);
        x = gx(fmaf(4.f, pdiff(E, W), pdiff(NE, NW) + pdiff(SE, SW)));
        y = gy(fmaf(4.f, pdiff(N, Sv), pdiff(NE, SE) + pdiff(NW, SW)));
    } else {
        x = 0.5f * pdiff(E, W);
        y = 0.5f * pdiff(N, Sv);
    }
    U[(size_t)UW_GP * qs + c] = x;
    U[(size_t)(UW_GP + 1) * qs + c] = y;
}

// Upwind reconstruction and fluxes of the west x-face (XF) or the south y-face of every
// cell n, between o (west / below) and n; the face at the origin, the cells' centres at
// -+1/2 along the normal (unit cells: every offset is exact).
template <int MODEL, bool XF>
__device__ __forceinline__ void uw_face(const P32 &P, const S32 &S, float *U, size_t co, size_t cn) {
    const size_t qs = S.qs;
    float av[6];
#pragma unroll
    for (int a = 0; a < 6; ++a) av[a] = 0.5f * (U[(size_t)(UW_A + a) * qs + co] + U[(size_t)(UW_A + a) * qs + cn]);
    const float2 po = phi_at(S, co), pn = phi_at(S, cn);
    const float avg = 0.5f * (po.x + pn.x), hdn = 0.5f * pdiff(pn, po);
    const float2 gpo = mk2(U[(size_t)UW_GP * qs + co], U[(size_t)(UW_GP + 1) * qs + co]);
    const float2 gpn = mk2(U[(size_t)UW_GP * qs + cn], U[(size_t)(UW_GP + 1) * qs + cn]);
    // cell u's value of direction q extrapolated by (dx, dy), its phi part relative to avg
    // (phis = phi_u - avg)
    auto ext = [&](int q, size_t cu, float dx, float dy, float phis, float2 gp) -> float2 {
        const float2 b = mk2(U[(size_t)(UW_B + q) * qs + cu], U[(size_t)(UW_B + 9 + q) * qs + cu]);
        const float2 gx = mk2(U[(size_t)(UW_GX + q) * qs + cu], U[(size_t)(UW_GX + 9 + q) * qs + cu]);
        const float2 gy = mk2(U[(size_t)(UW_GY + q) * qs + cu], U[(size_t)(UW_GY + 9 + q) * qs + cu]);
        const float2 x = fma2(mk2(dy, dy), gy, fma2(mk2(dx, dx), gx, b));
        const float wp = fmaf(dy, gp.y, fmaf(dx, gp.x, phis));
        return mk2(x.x, fmaf((float)d2q9_w(q), wp, x.y));
    };
    float2 bh[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const float xu = (float)d2q9_xu(q), xv = (float)d2q9_xv(q);
        const float sx = -P.hDt * xu, sy = -P.hDt * xv;
        const float dxo = XF ? 0.5f + sx : sx, dyo = XF ? sy : 0.5f + sy;
        const float dxn = XF ? sx - 0.5f : sx, dyn = XF ? sy : sy - 0.5f;
        const int s = XF ? d2q9_xu(q) : d2q9_xv(q);
        if (s > 0) {
            bh[q] = ext(q, co, dxo, dyo, -hdn, gpo);
        } else if (s < 0) {
            bh[q] = ext(q, cn, dxn, dyn, hdn, gpn);
        } else {
            bh[q] = mul2(mk2(0.5f, 0.5f), add2(ext(q, co, dxo, dyo, -hdn, gpo), ext(q, cn, dxn, dyn, hdn, gpn)));
        }
    }
    float2 F[6];
    face_state_flux<MODEL, XF, float>(P, bh, av, avg, 0, F);
    const int base = XF ? UW_XF : UW_YF;
#pragma unroll
    for (int s = 0; s < 6; ++s) {
        U[(size_t)(base + 2 * s) * qs + cn] = F[s].x;
        U[(size_t)(base + 2 * s + 1) * qs + cn] = F[s].y;
    }
}

// the west x-face and the south y-face of every cell, one thread both (the cell's own
// values, read by both, come from the cache the second time: half the DRAM reads of one
// launch slice per face direction)
template <int MODEL>
__global__ void __launch_bounds__(UBX *UBY) k_uw32_faces(P32 P, S32 S, float *U) {
    Cells k;
    if (!cell_of(P, k)) return;
    uw_face<MODEL, true>(P, S, U, at(P, k.j, k.im), k.c);
    uw_face<MODEL, false>(P, S, U, at(P, k.jm, k.i), k.c);
}

// finite-volume update of every cell from its four faces' fluxes
template <int MODEL>
__global__ void __launch_bounds__(UBX *UBY) k_uw32_update(P32 P, S32 S, const float *U) {
    Cells k;
    if (!cell_of(P, k)) return;
    const size_t qs = S.qs, c = k.c;
    float2 Pq[9], inc[9], FW[6], FE[6], FS[6], FN[6], dn[9];
    float sfz;
    load_cell<MODEL>(S, c, Pq, sfz);
#pragma unroll
    for (int q = 0; q < 9; ++q) inc[q] = mk2(U[(size_t)(UW_INC + q) * qs + c], U[(size_t)(UW_INC + 9 + q) * qs + c]);
    const size_t cE = at(P, k.j, k.ip), cN = at(P, k.jp, k.i);
#pragma unroll
    for (int s = 0; s < 6; ++s) {
        FW[s] = mk2(U[(size_t)(UW_XF + 2 * s) * qs + c], U[(size_t)(UW_XF + 2 * s + 1) * qs + c]);
        FE[s] = mk2(U[(size_t)(UW_XF + 2 * s) * qs + cE], U[(size_t)(UW_XF + 2 * s + 1) * qs + cE]);
        FS[s] = mk2(U[(size_t)(UW_YF + 2 * s) * qs + c], U[(size_t)(UW_YF + 2 * s + 1) * qs + c]);
        FN[s] = mk2(U[(size_t)(UW_YF + 2 * s) * qs + cN], U[(size_t)(UW_YF + 2 * s + 1) * qs + cN]);
    }
    const float half_dtv = 0.5f * P.dtV;
    const float px = half_dtv * pdiff(phi_at(S, at(P, k.j, k.im)), phi_at(S, cE));
    const float py = half_dtv * pdiff(phi_at(S, at(P, k.jm, k.i)), phi_at(S, cN));
    float dphi;
    update_cell<float>(P, Pq, inc, FW, FE, FS, FN, px, py, dn, dphi);
    S.odf[c] = dn[0].x;
#pragma unroll
    for (int q = 1; q < 9; ++q) {
        S.odf[(size_t)q * qs + c] = dn[q].x;
        S.odg[(size_t)(q - 1) * qs + c] = dn[q].y;
    }
    const float2 pn = phi_add(phi_at(S, c), dphi);
    S.ophi[c] = pn.x;
    S.ophi[qs + c] = pn.y;
}

template <int MODEL>
static cudaError_t launch_uw32_t(const P32 &P, const S32 &S, float *U, int first, cudaStream_t st) {
    const dim3 blk(UBX, UBY), grd((P.nx + UBX - 1) / UBX, (P.ny + UBY - 1) / UBY);
    k_uw32_collide<MODEL><<<grd, blk, 0, st>>>(P, S, U, first);
    k_uw32_grad<<<dim3(grd.x, grd.y, UW_GRAD_SLICES), blk, 0, st>>>(P, S, U);
    k_uw32_faces<MODEL><<<grd, blk, 0, st>>>(P, S, U);
    k_uw32_update<MODEL><<<grd, blk, 0, st>>>(P, S, U);
    return cudaGetLastError();
}

// One UW step of a periodic FP32 Allen-Cahn case: reads the copy S.df.., writes S.odf..
// (the caller swaps them); U: UW_PLANES scratch planes of S.qs floats.
cudaError_t launch_uw32(const P32 &P, const S32 &S, float *U, int first, cudaStream_t st, int64_t *launches) {
    if (P.walls || !U) return cudaErrorInvalidValue;
    const cudaError_t e = P.model == AC ? launch_uw32_t<AC>(P, S, U, first, st) : launch_uw32_t<HCZ>(P, S, U, first, st);
    if (e == cudaSuccess) *launches += 4;
    return e;
}

}  // namespace f32
}  // namespace dugks
