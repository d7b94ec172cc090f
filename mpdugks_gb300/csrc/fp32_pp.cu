// FP32 deviation-storage step of the pseudopotential models (D2Q9PP, D2V16).
//
// The reference's face force reads the face psi of the neighbouring faces of
// the same step (Ark/Cpp/PseudoP.cpp:39-46, Jacobi semantics: all face psi
// first, then the face forces), so the step keeps four passes like the FP64
// path: collision (with the cell force from the psi of the previous update),
// face pass 1 (reconstruction, face moments, face psi), face pass 2 (face
// force, equilibrium, He-Shan-Doolen source, flux) and the update (with the
// cell macros, pressure and psi).
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
// (Fusing face pass 2 with the update, the fluxes of a tile in shared memory and the
// face reconstruction recomputed instead of stored, ran slower: 0.55 against 0.46 ms
// per D2V16 step at 1024^2, 128 registers and two blocks per SM.)
#include <cuda_runtime.h>

#include <cstdint>

#include "dugks_device.cuh"
#include "fp32_math.cuh"
#include "fp32_state.cuh"

namespace dugks {
namespace f32 {

// Equilibrium parts de_q = eq_q(rho, u, v) - e_q rho (zero at rest).
template <int MODEL>
__device__ __forceinline__ void pp_deq(const PPP &P, float rho, float u, float v, float *de) {
    if (MODEL == PP16) {
        // Macro16 (Ark/Lib/D2V16.cpp:125-145) at T = T0, p = rho RT, minus its value at
        // (rho, 0, 0) (at rest the moments are linear in rho); times the case's inverse
        // moment matrix (Ark/Lib/D2V16.cpp:34-52), read through the read-only path (every
        // lane of a warp reads the same entry)
        const float RT = P.RT, u2 = u * u, v2 = v * v, s2 = u2 + v2;
        float M[16];
        M[0] = 0.f;
        M[1] = rho * u;
        M[2] = rho * v;
        M[3] = rho * s2;
        M[4] = M[1] * v;
        M[5] = rho * u2;
        M[6] = rho * v2;
        M[7] = M[1] * (5.f * RT + s2);
        M[8] = M[2] * (5.f * RT + s2);
        M[9] = M[1] * (3.f * RT + u2);
        M[10] = M[2] * (3.f * RT + v2);
        M[11] = M[2] * (RT + u2);
        M[12] = M[1] * (RT + v2);
        M[13] = (7.f * RT + s2) * M[4];
        M[14] = rho * RT * (8.f * u2 + v2) + rho * u2 * s2;
        M[15] = rho * RT * (8.f * v2 + u2) + rho * v2 * s2;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            float s = 0.f;
#pragma unroll
            for (int k = 1; k < 16; ++k) s = fmaf(__ldg(P.iM16 + j * 16 + k), M[k], s);
            de[j] = s;
        }
    } else {
        // D2Q9PP (Ark/Lib/D2Q9PP.cpp:51-62): w rho (1 + u1 + u1^2/2 - |u|^2 lambda) - w rho
        const float uu = u * u + v * v;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const float u1 = (sxf(d2q9_xu(q), u) + sxf(d2q9_xv(q), v)) * P.invRT;
            de[q] = P.w9[q] * (rho * (u1 + 0.5f * u1 * u1 - uu * P.Lambda0));
        }
    }
}

// ---- float-float arithmetic: a value is the unevaluated sum hi + lo of two
// floats.  TwoSum (Knuth, TAOCP vol. 2, 4.2.2), FastTwoSum (Dekker 1971), the
// product error by fma, the cascaded sum Sum2 (Ogita, Rump and Oishi 2005) and a
// two-step long division as in Bailey's double-double arithmetic: about 44
// significant bits, for the moment sums and the equation of state that the FP64
// path evaluates in double (the FP64 units of this GPU are ~1/60 of its FP32
// rate, and these were most of this path's time).  Products that feed a TwoSum
// use __fmul_rn so that no fma contraction changes them.
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF two_sum(float a, float b) {
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ FF fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ void ff_acc(FF &s, float x) {  // Sum2 step: s += x
    const FF t = two_sum(s.hi, x);
    s.hi = t.hi;
    s.lo = __fadd_rn(s.lo, t.lo);
}
__device__ __forceinline__ void ff_acc_prod(FF &s, float a, float b) {  // s += a b, the product exactly
    const float p = __fmul_rn(a, b);
    ff_acc(s, p);
    s.lo = __fadd_rn(s.lo, fmaf(a, b, -p));
}
__device__ __forceinline__ FF ff_neg(FF a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    FF t = two_sum(a.hi, b.hi);
    t.lo = __fadd_rn(t.lo, __fadd_rn(a.lo, b.lo));
    return two_sum(t.hi, t.lo);
}
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ FF ff_div(FF a, FF b) {
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const FF r = ff_add(a, ff_neg(ff_mul(b, FF{q1, 0.f})));
    return fast_two_sum(q1, __fdiv_rn(__fadd_rn(r.hi, r.lo), b.hi));
}
__device__ __forceinline__ FF ff_norm(FF a) { return two_sum(a.hi, a.lo); }

// Carnahan-Starling pressure (Ark/Lib/nonidealEoS.h:114-118) of the density r:
// r R0 T (1 + r + r^2 - r^3) / (1 - r)^3 - a r^2
__device__ __forceinline__ FF cs_p(const PPP &P, FF r) {
    const FF one{1.f, 0.f};
    const FF r2 = ff_mul(r, r), r3 = ff_mul(r2, r);
    const FF num = ff_add(ff_add(ff_add(one, r), r2), ff_neg(r3));
    const FF om = ff_add(one, ff_neg(r));
    const FF den = ff_mul(ff_mul(om, om), om);
    return ff_add(ff_mul(ff_mul(r, FF{P.rtcs_hi, P.rtcs_lo}), ff_div(num, den)),
                  ff_neg(ff_mul(FF{P.acs_hi, P.acs_lo}, r2)));
}
// calcPsi (Ark/Header/Macroscopic.h:64-68): G = sign(p - rho RT), psi = sqrt(2 (p - rho RT) / G)
// psi as a float-float pair (hi, lo): the square root's head and the correction
// (x - hi^2) / (2 hi) of its residual (hi^2 exactly by fma); the gradient stencil of
// psi then differences pairs, which matters where grad psi is small against psi
__device__ __forceinline__ void cs_psi(const PPP &P, FF rho, FF p, float &scg, float &psi, float &psil) {
    const FF g = ff_add(p, ff_neg(ff_mul(rho, FF{P.rt_hi, P.rt_lo})));
    const float G = (float)((g.hi > 0.f) - (g.hi < 0.f));
    scg = G;
    const float xh = 2.f * g.hi * G, xl = 2.f * g.lo * G;  // G = +-1: exact
    psi = sqrtf(xh);
    psil = psi > 0.f ? __fdiv_rn(fmaf(-psi, psi, xh) + xl, 2.f * psi) : 0.f;
}
__device__ __forceinline__ double ff_to_double(FF a) { return (double)a.hi + (double)a.lo; }


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
    const float2 E = at(j, ip), W = at(j, im), N = at(jp, i), S = at(jm, i);
    const float2 NE = at(jp, ip), NW = at(jp, im), SE = at(jm, ip), SW = at(jm, im);
    gx = (4.f * pdiff(E, W) + (pdiff(NE, NW) + pdiff(SE, SW))) * P.inv_6_2dx;
    gy = (4.f * pdiff(N, S) + (pdiff(NE, SE) + pdiff(NW, SW))) * P.inv_6_2dy;
}

// Collision pre-step: cell force F = -G psi grad psi (Ark/Cpp/PseudoP.cpp:31-38, from the
// previous update's psi) when do_msrc, equilibrium, source; f-bar-plus as the remainder
// B_q - e_q rho = g_q + (1 - a)(de_q - g_q) + c S_q.
template <int MODEL>
__global__ void __launch_bounds__(256) k_pp32_collide(PPP P, PPS S, int do_msrc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= P.nx || j >= P.ny) return;
    constexpr int Q = MODEL == PP16 ? 16 : 9;
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
    const float rho = (float)S.rho[c];
    const float U = (float)S.U[c], V = (float)S.V[c];
    float de[Q];
    pp_deq<MODEL>(P, rho, U, V, de);
    const float tau = P.Tau0;
    const float aBP = (2.f * tau - P.hDt) / (2.f * tau + P.dt), bBP = 1.f - aBP, cBP = tau * bBP;
    const float inv = 1.f / (rho * P.RT);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float eq = fmaf(P.erest[q], rho, de[q]);
        const float So = (fx * (P.xi_u[q] - U) + fy * (P.xi_v[q] - V)) * eq * inv;
        const size_t o = (size_t)q * S.qs + c;
        const float g = S.df[o];
        S.bf[o] = g + (bBP * (de[q] - g) + cBP * So);
    }
}

// Face pass 1 (x faces: blockIdx.z = 0, y faces: 1): half-step reconstruction,
// face moments with the previous face force, face pressure and psi
// (Ark/Lib/D2Q9PP.cpp:110-136, Ark/Cpp/PseudoP.cpp:23-30).  The face values are
// stored relative to e_q times the face average of rho: the reconstruction of the
// remainders plus e_q (L_q(rho) - avg), L_q(rho) the same reconstruction applied to the
// FP64 density.
template <int MODEL>
__global__ void __launch_bounds__(256) k_pp32_faces1(PPP P, PPS S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool xf = blockIdx.z == 0;
    if (i >= P.nx || j >= P.ny) return;
    constexpr int Q = MODEL == PP16 ? 16 : 9;
    const int nx = P.nx, ny = P.ny, pitch = P.pitch;
    const int im = wrapi(i - 1, nx), ip = wrapi(i + 1, nx), jm = wrapi(j - 1, ny), jp = wrapi(j + 1, ny);
    const size_t c = (size_t)j * pitch + i;
    auto rh = [&](int jj, int ii) { return S.rho[(size_t)jj * pitch + ii]; };
    // the density's reconstruction: face average and hDt times its gradient
    double ravg, hgx, hgy;
    if (xf) {
        ravg = 0.5 * (rh(j, im) + rh(j, i));
        hgx = (double)P.hDt * ((rh(j, im) - rh(j, i)) * (double)P.r_ndx);
        hgy = (double)P.hDt * ((0.5 * ((rh(jp, i) - rh(jm, i)) + (rh(jp, im) - rh(jm, im)))) * (double)P.r_2dy);
    } else {
        ravg = 0.5 * (rh(jm, i) + rh(j, i));
        hgx = (double)P.hDt * ((0.5 * ((rh(j, im) - rh(j, ip)) + (rh(jm, im) - rh(jm, ip)))) * (double)P.r_n2dx);
        hgy = (double)P.hDt * ((rh(jm, i) - rh(j, i)) * (double)P.r_ndy);
    }
    const float hgxf = (float)hgx, hgyf = (float)hgy;
    // face moments as float-float sums
    FF sR{0.f, 0.f}, su{0.f, 0.f}, sv{0.f, 0.f};
    float *B = xf ? S.xb : S.yb;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float *F = S.bf + (size_t)q * S.qs;
        auto at = [&](int jj, int ii) { return F[(size_t)jj * pitch + ii]; };
        float o, n, gx, gy;
        if (xf) {  // between (i-1, j) and (i, j)
            o = at(j, im);
            n = at(j, i);
            gy = (0.5f * ((at(jp, i) - at(jm, i)) + (at(jp, im) - at(jm, im)))) * P.r_2dy;
            gx = (o - n) * P.r_ndx;
        } else {  // between (i, j-1) and (i, j)
            o = at(jm, i);
            n = at(j, i);
            gx = (0.5f * ((at(j, im) - at(j, ip)) + (at(jm, im) - at(jm, ip)))) * P.r_n2dx;
            gy = (o - n) * P.r_ndy;
        }
        float b = 0.5f * (o + n) - P.hDt * (gx * P.xi_u[q] + gy * P.xi_v[q]);
        b = fmaf(-P.erest[q], hgxf * P.xi_u[q] + hgyf * P.xi_v[q], b);
        B[(size_t)q * S.qs + c] = b;
        ff_acc(sR, b);
        ff_acc_prod(su, b, P.xi_u[q]);
        ff_acc_prod(sv, b, P.xi_v[q]);
    }
    sR = ff_norm(sR);
    const float rah = (float)ravg;
    const FF R = ff_add(FF{rah, (float)(ravg - (double)rah)}, sR);
    const float Rf = R.hi;
    float U = __fadd_rn(su.hi, su.lo) / Rf, V = __fadd_rn(sv.hi, sv.lo) / Rf;
    U += 0.5f * P.hDt * (xf ? S.xFx : S.yFx)[c] / Rf;
    V += 0.5f * P.hDt * (xf ? S.xFy : S.yFy)[c] / Rf;
    const FF p = cs_p(P, R);
    float scg, psi, psil;
    cs_psi(P, R, p, scg, psi, psil);
    (xf ? S.xpsl : S.ypsl)[c] = psil;
    (xf ? S.xr : S.yr)[c] = __fadd_rn(sR.hi, sR.lo);  // face rho - avg(rho)
    (xf ? S.xu : S.yu)[c] = U;
    (xf ? S.xv : S.yv)[c] = V;
    (xf ? S.xg : S.yg)[c] = scg;
    (xf ? S.xps : S.yps)[c] = psi;
}

// Face pass 2: face force from the face-psi stencil (Ark/Cpp/PseudoP.cpp:39-46,
// Ark/Lib/GradSchemeBasic.h:181-208), equilibrium, source and flux xi.n of the face
// values relative to e_q avg(rho).
template <int MODEL>
__global__ void __launch_bounds__(256) k_pp32_faces2(PPP P, PPS S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool xf = blockIdx.z == 0;
    if (i >= P.nx || j >= P.ny) return;
    constexpr int Q = MODEL == PP16 ? 16 : 9;
    const size_t c = (size_t)j * P.pitch + i;
    float gx, gy;
    iso_grad(P, xf ? S.xps : S.yps, xf ? S.xpsl : S.ypsl, i, j, gx, gy);
    const float k = -(xf ? S.xg : S.yg)[c] * (xf ? S.xps : S.yps)[c];
    const float Fx = gx * k, Fy = gy * k;
    (xf ? S.xFx : S.yFx)[c] = Fx;
    (xf ? S.xFy : S.yFy)[c] = Fy;
    const float dr = (xf ? S.xr : S.yr)[c];
    const size_t co = xf ? (size_t)j * P.pitch + wrapi(i - 1, P.nx) : (size_t)wrapi(j - 1, P.ny) * P.pitch + i;
    const float R = (float)(0.5 * (S.rho[co] + S.rho[c]) + (double)dr);
    const float U = (xf ? S.xu : S.yu)[c], V = (xf ? S.xv : S.yv)[c];
    float de[Q];
    pp_deq<MODEL>(P, R, U, V, de);
    const float tauh = P.Tau0;
    const float ah = 2.f * tauh / (2.f * tauh + P.hDt), bh = 1.f - ah, ch = tauh * bh;
    const float inv = 1.f / (R * P.RT);
    const float *__restrict__ B = xf ? S.xb : S.yb;
    float *out = xf ? S.xfl : S.yfl;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float eq = fmaf(P.erest[q], R, de[q]);
        const float So = (Fx * (P.xi_u[q] - U) + Fy * (P.xi_v[q] - V)) * eq * inv;
        const float heq = fmaf(P.erest[q], dr, de[q]);  // eq - e_q avg(rho)
        const float b = B[(size_t)q * S.qs + c];
        const float t = heq + ah * (b - heq) + ch * So;
        out[(size_t)q * S.qs + c] = t * (xf ? P.xi_u[q] : P.xi_v[q]);
    }
}

// Update (Ark/Cpp/DUGKS2DSolver.cpp:748-792) and cell macros (Ark/Lib/D2Q9PP.cpp:89-109):
//   rho_new = rho + drho, drho = dt/V sum_q (net face flux of q),
//   g_q,new = g_q + 4/3 (b_q - g_q) + dt/V (net flux of q)
//             + e_q (xi_q,x px + xi_q,y py) - e_q drho,
// px = dt/V (rho_W - rho_E)/2, py = dt/V (rho_S - rho_N)/2 (the e_q avg(rho) flux
// divergence on unit cells, from the FP64 density); U, V, p, psi from float-float
// sums, rho in FP64.
template <int MODEL>
__global__ void __launch_bounds__(256) k_pp32_update(PPP P, PPS S, uint32_t step) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= P.nx || j >= P.ny) return;
    constexpr int Q = MODEL == PP16 ? 16 : 9;
    const int pitch = P.pitch;
    const int ip = wrapi(i + 1, P.nx), im = wrapi(i - 1, P.nx), jn = wrapi(j + 1, P.ny), js = wrapi(j - 1, P.ny);
    const size_t c = (size_t)j * pitch + i, cE = (size_t)j * pitch + ip, cN = (size_t)jn * pitch + i;
    const double rho = S.rho[c];
    const float px = (float)(0.5 * (double)P.dtV * (S.rho[(size_t)j * pitch + im] - S.rho[cE]));
    const float py = (float)(0.5 * (double)P.dtV * (S.rho[(size_t)js * pitch + i] - S.rho[cN]));
    float sq[Q];
    FF sd{0.f, 0.f};
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const size_t o = (size_t)q * S.qs;
        float s = 0.f;
        s += -S.xfl[o + cE];
        s += -S.yfl[o + cN];
        s += S.xfl[o + c];
        s += S.yfl[o + c];
        sq[q] = s;
        ff_acc(sd, s);
    }
    const double drho = (double)P.dtV * ((double)sd.hi + (double)sd.lo);
    const float drf = (float)drho;
    const double rho_n = rho + drho;
    FF su{0.f, 0.f}, sv{0.f, 0.f};
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const size_t o = (size_t)q * S.qs;
        const float g = S.df[o + c];
        float inc = fmaf(P.aTP, S.bf[o + c] - g, P.dtV * sq[q]);
        inc = fmaf(P.erest[q], (P.xi_u[q] * px + P.xi_v[q] * py) - drf, inc);
        const float gn = g + inc;
        S.df[o + c] = gn;
        ff_acc_prod(su, gn, P.xi_u[q]);
        ff_acc_prod(sv, gn, P.xi_v[q]);
    }
    const float rh = (float)rho_n;
    const FF R{rh, (float)(rho_n - (double)rh)};
    float U = __fadd_rn(su.hi, su.lo) / rh, V = __fadd_rn(sv.hi, sv.lo) / rh;
    U += P.hDt * S.Fx[c] / rh;
    V += P.hDt * S.Fy[c] / rh;
    const FF p = cs_p(P, R);
    float scg, psi, psil;
    cs_psi(P, R, p, scg, psi, psil);
    S.rho_o[c] = rho_n;
    S.psil[c] = psil;
    S.U[c] = U;
    S.V[c] = V;
    S.p[c] = ff_to_double(p);
    S.scg[c] = scg;
    S.psi[c] = psi;
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
    k_pp32_collide<MODEL><<<grd, blk, 0, st>>>(P, S, do_msrc);
    k_pp32_faces1<MODEL><<<grf, blk, 0, st>>>(P, S);
    k_pp32_faces2<MODEL><<<grf, blk, 0, st>>>(P, S);
    k_pp32_update<MODEL><<<grd, blk, 0, st>>>(P, S, step);
    *launches += 4;
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
