// Per-cell and per-face arithmetic of the FP32 pseudopotential step (D2Q9PP, D2V16),
// shared by the three-pass kernels (fp32_pp.cu) and the single-pass streaming kernel
// (fp32_pp_stream.cu), so both evaluate the same expressions.  Storage: the density in
// FP64, f as the FP32 remainders g_q = f_q - e_q rho (fp32_pp.cu has the derivation).
#pragma once
#include <cuda_runtime.h>

#include "dugks_device.cuh"
#include "fp32_math.cuh"
#include "fp32_state.cuh"

namespace dugks {
namespace f32 {

template <int MODEL>
struct PPQ {
    static constexpr int Q = MODEL == PP16 ? 16 : 9;
};

// The velocity set as integers times the lattice speed (D2V16: Ark/Lib/D2V16.cpp:53-66,
// D2Q9: Ark/Lib/D2Q9.h:86-88) and each direction's opposite
template <int MODEL>
__host__ __device__ constexpr int lat_u(int q) {
    return MODEL == PP16 ? (q == 0 || q == 4 || q == 7 ? 1 : q == 2 || q == 5 || q == 6 ? -1 : q == 8 || q == 12 || q == 15 ? 2
                                                                                        : q == 10 || q == 13 || q == 14 ? -2 : 0)
                         : d2q9_xu(q);
}
template <int MODEL>
__host__ __device__ constexpr int lat_v(int q) {
    return MODEL == PP16 ? (q == 1 || q == 4 || q == 5 ? 1 : q == 3 || q == 6 || q == 7 ? -1 : q == 9 || q == 12 || q == 13 ? 2
                                                                                        : q == 11 || q == 14 || q == 15 ? -2 : 0)
                         : d2q9_xv(q);
}
template <int MODEL>
__host__ __device__ constexpr int lat_opp(int q) {
    return MODEL == PP16 ? d2v16_opp(q) : d2q9_bb(q);
}

// Equilibrium parts de_q = eq_q(rho, u, v) - e_q rho (zero at rest).
template <int MODEL>
__device__ __forceinline__ void pp_deq(const PPP &P, float rho, float u, float v, float *de) {
    if (MODEL == PP16) {
        // Macro16 (Ark/Lib/D2V16.cpp:125-145) at T = T0, p = rho RT, minus its value at
        // (rho, 0, 0) (at rest the moments are linear in rho); times the case's inverse
        // moment matrix (Ark/Lib/D2V16.cpp:34-52), a kernel parameter
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
        // row j' (the opposite direction of j) holds row j's entries of the even moments and
        // the negated entries of the odd ones, and the axis rings' rows have fixed zeros
        // (d2v16_odd_moment, d2v16_entry): per opposite pair the even and odd partial sums,
        // de_j = E + O, de_j' = E - O
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int jo = lat_opp<PP16>(j);
            if (jo < j) continue;
            float E = 0.f, O = 0.f;
#pragma unroll
            for (int k = 1; k < 16; ++k) {
                if (!d2v16_entry(j, k)) continue;
                if (d2v16_odd_moment(k)) O = fmaf(P.iM16[j][k], M[k], O);
                else E = fmaf(P.iM16[j][k], M[k], E);
            }
            de[j] = E + O;
            de[jo] = E - O;
        }
    } else {
        // D2Q9PP (Ark/Lib/D2Q9PP.cpp:51-62): w rho (1 + u1 + u1^2/2 - |u|^2 lambda) - w rho;
        // every rounding written out, so that each kernel including this evaluates it alike
        const float uu = fmaf(u, u, __fmul_rn(v, v));
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const float u1 = __fmul_rn(__fadd_rn(sxf(d2q9_xu(q), u), sxf(d2q9_xv(q), v)), P.invRT);
            const float t = fmaf(__fmul_rn(0.5f, u1), u1, u1);
            de[q] = __fmul_rn(P.w9[q], __fmul_rn(rho, fmaf(-uu, P.Lambda0, t)));
        }
    }
}

// ---- float-float arithmetic: a value is the unevaluated sum hi + lo of two
// floats.  TwoSum (Knuth, TAOCP vol. 2, 4.2.2), FastTwoSum (Dekker 1971), the
// product error by fma, the cascaded sum Sum2 (Ogita, Rump and Oishi 2005) and a
// two-step long division as in Bailey's double-double arithmetic: about 44
// significant bits, for the moment sums and the equation of state that the FP64
// path evaluates in double (the FP64 units of this GPU are ~1/60 of its FP32
// rate, and these were most of this path's time).
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

// n b as an exact float for the integer n in {-2, ..., 2}
__device__ __forceinline__ float times_small(int n, float b) { return n == 1 ? b : n == -1 ? -b : n == 2 ? 2.f * b : -2.f * b; }

// First moments sum_q xi_q b_q (x, y) as float-float: over the opposite pairs (q, q') of
// n_q (b_q - b_q'), n_q = xi_q / speed an integer (each term exact scaling of one rounded
// difference, zero components skipped), then times the lattice speed as a pair
template <int MODEL>
__device__ __forceinline__ void pp_first_moments(const PPP &P, const float (&b)[PPQ<MODEL>::Q], FF &su, FF &sv) {
    constexpr int Q = PPQ<MODEL>::Q;
    FF ax{0.f, 0.f}, ay{0.f, 0.f};
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int qo = lat_opp<MODEL>(q);
        if (qo <= q) continue;  // each pair once, from its lower index; the rest direction has none
        const float d = __fsub_rn(b[q], b[qo]);
        const int nu = lat_u<MODEL>(q), nv = lat_v<MODEL>(q);
        if (nu != 0) ff_acc(ax, times_small(nu, d));
        if (nv != 0) ff_acc(ay, times_small(nv, d));
    }
    const FF c{P.lat_hi, P.lat_lo};
    su = ff_mul(ff_norm(ax), c);
    sv = ff_mul(ff_norm(ay), c);
}



// 8-neighbour isotropic gradient (Ark/Lib/GradSchemeBasic.h:153-208) from the float-float
// pairs of the eight neighbours, by pair differences
__device__ __forceinline__ void pp_iso_grad(const PPP &P, float2 E, float2 W, float2 N, float2 S, float2 NE,
                                            float2 NW, float2 SE, float2 SW, float &gx, float &gy) {
    gx = (4.f * pdiff(E, W) + (pdiff(NE, NW) + pdiff(SE, SW))) * P.inv_6_2dx;
    gy = (4.f * pdiff(N, S) + (pdiff(NE, SE) + pdiff(NW, SW))) * P.inv_6_2dy;
}

// The He-Shan-Doolen projections (xi_q - u).F of the directions, by opposite pairs: with
// d = xi_q.F and w = u.F, (xi_q - u).F = d - w and (xi_q' - u).F = -d - w (xi_q' = -xi_q);
// a rest direction (D2Q9PP's 0) has -w.
template <int MODEL>
__device__ __forceinline__ void pp_src_proj(const PPP &P, float fx, float fy, float U, float V,
                                            float (&pr)[PPQ<MODEL>::Q]) {
    constexpr int Q = PPQ<MODEL>::Q;
    const float w = fmaf(fx, U, fy * V);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int qo = lat_opp<MODEL>(q);
        if (qo < q) continue;
        if (qo == q) {
            pr[q] = -w;
            continue;
        }
        const float d = fmaf(fx, P.xi_u[q], fy * P.xi_v[q]);
        pr[q] = d - w;
        pr[qo] = -d - w;
    }
}

// Collision pre-step of one cell: f-bar-plus as the remainder
// B_q - e_q rho = g_q + (1 - a)(de_q - g_q) + c S_q, S the He-Shan-Doolen source of the
// cell force (fx, fy).
template <int MODEL>
__device__ __forceinline__ void pp_collide(const PPP &P, const float (&g)[PPQ<MODEL>::Q], float rho, float U, float V,
                                           float fx, float fy, float (&bf)[PPQ<MODEL>::Q]) {
    constexpr int Q = PPQ<MODEL>::Q;
    float de[Q];
    pp_deq<MODEL>(P, rho, U, V, de);
    const float tau = P.Tau0;
    const float aBP = (2.f * tau - P.hDt) / (2.f * tau + P.dt), bBP = 1.f - aBP, cBP = tau * bBP;
    const float inv = 1.f / (rho * P.RT);
    float pr[Q];
    pp_src_proj<MODEL>(P, fx, fy, U, V, pr);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float eq = fmaf(P.erest[q], rho, de[q]);
        const float So = pr[q] * eq * inv;
        bf[q] = g[q] + (bBP * (de[q] - g[q]) + cBP * So);
    }
}

// Face pass 1 of one face (XF: an x face between o = west and n = east cell, else a y face
// between o = below and n = above): the half-step reconstruction relative to e_q times the
// face average of rho, from the f-bar-plus remainders of the two cells (o, n) and the sums
// tn, to of their tangential differences ((t+) - (t-) of n and of o: x face rows +-1, y face
// columns -1 minus +1); ravg, hgx, hgy: the density's face average and hDt times its
// gradient (FP64); (fxp, fyp): the face force of the previous step.  Out: b, the face
// velocity, the face density relative to ravg (dr) and the face psi pair and sign.
struct PPFace {
    float U, V, dr, psi, psil, scg;
};
template <int MODEL, bool XF>
__device__ __forceinline__ PPFace pp_face1(const PPP &P, const float (&o)[PPQ<MODEL>::Q],
                                           const float (&n)[PPQ<MODEL>::Q], const float (&tn)[PPQ<MODEL>::Q],
                                           const float (&to)[PPQ<MODEL>::Q], double ravg, double hgx, double hgy,
                                           float fxp, float fyp, float (&b)[PPQ<MODEL>::Q]) {
    constexpr int Q = PPQ<MODEL>::Q;
    const float hgxf = (float)hgx, hgyf = (float)hgy;
    FF sR{0.f, 0.f}, su{0.f, 0.f}, sv{0.f, 0.f};
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        float gx, gy;
        if (XF) {
            gy = (0.5f * (tn[q] + to[q])) * P.r_2dy;
            gx = (o[q] - n[q]) * P.r_ndx;
        } else {
            gx = (0.5f * (tn[q] + to[q])) * P.r_n2dx;
            gy = (o[q] - n[q]) * P.r_ndy;
        }
        float bq = 0.5f * (o[q] + n[q]) - P.hDt * (gx * P.xi_u[q] + gy * P.xi_v[q]);
        bq = fmaf(-P.erest[q], hgxf * P.xi_u[q] + hgyf * P.xi_v[q], bq);
        b[q] = bq;
        ff_acc(sR, bq);
    }
    pp_first_moments<MODEL>(P, b, su, sv);
    sR = ff_norm(sR);
    const float rah = (float)ravg;
    const FF R = ff_add(FF{rah, (float)(ravg - (double)rah)}, sR);
    const float Rf = R.hi;
    PPFace f;
    f.U = __fadd_rn(su.hi, su.lo) / Rf;
    f.V = __fadd_rn(sv.hi, sv.lo) / Rf;
    f.U += 0.5f * P.hDt * fxp / Rf;
    f.V += 0.5f * P.hDt * fyp / Rf;
    const FF p = cs_p(P, R);
    cs_psi(P, R, p, f.scg, f.psi, f.psil);
    f.dr = __fadd_rn(sR.hi, sR.lo);  // face rho - avg(rho)
    return f;
}

// Face pass 2 of one face: equilibrium, source of the face force (fx, fy) and the flux
// xi.n of the face values relative to e_q avg(rho); R the face density.
template <int MODEL, bool XF>
__device__ __forceinline__ void pp_face2(const PPP &P, const float (&b)[PPQ<MODEL>::Q], float R, const PPFace &f,
                                         float fx, float fy, float (&out)[PPQ<MODEL>::Q]) {
    constexpr int Q = PPQ<MODEL>::Q;
    float de[Q];
    pp_deq<MODEL>(P, R, f.U, f.V, de);
    const float tauh = P.Tau0;
    const float ah = 2.f * tauh / (2.f * tauh + P.hDt), bh = 1.f - ah, ch = tauh * bh;
    const float inv = 1.f / (R * P.RT);
    float pr[Q];
    pp_src_proj<MODEL>(P, fx, fy, f.U, f.V, pr);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float eq = fmaf(P.erest[q], R, de[q]);
        const float So = pr[q] * eq * inv;
        const float heq = fmaf(P.erest[q], f.dr, de[q]);  // eq - e_q avg(rho)
        const float t = heq + ah * (b[q] - heq) + ch * So;
        out[q] = t * (XF ? P.xi_u[q] : P.xi_v[q]);
    }
}

// Update of one cell (Ark/Cpp/DUGKS2DSolver.cpp:748-792) and its macros
// (Ark/Lib/D2Q9PP.cpp:89-109): fw, fe, fs, fn the fluxes of its west, east, south and
// north faces; rho and (px, py) = dt/V (rho_W - rho_E, rho_S - rho_N)/2 in FP64 / FP32;
// (fx, fy) the cell force of this step's collision.
struct PPCell {
    double rho, p;
    float U, V, psi, psil, scg;
};
template <int MODEL>
__device__ __forceinline__ PPCell pp_update(const PPP &P, float (&g)[PPQ<MODEL>::Q],
                                            const float (&bf)[PPQ<MODEL>::Q], const float (&fw)[PPQ<MODEL>::Q],
                                            const float (&fe)[PPQ<MODEL>::Q], const float (&fs)[PPQ<MODEL>::Q],
                                            const float (&fn)[PPQ<MODEL>::Q], double rho, float px, float py,
                                            float fx, float fy) {
    constexpr int Q = PPQ<MODEL>::Q;
    float sq[Q];
    FF sd{0.f, 0.f};
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        float s = 0.f;
        s += -fe[q];
        s += -fn[q];
        s += fw[q];
        s += fs[q];
        sq[q] = s;
        ff_acc(sd, s);
    }
    const double drho = (double)P.dtV * ((double)sd.hi + (double)sd.lo);
    const float drf = (float)drho;
    PPCell c;
    c.rho = rho + drho;
    FF su{0.f, 0.f}, sv{0.f, 0.f};
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        float inc = fmaf(P.aTP, bf[q] - g[q], P.dtV * sq[q]);
        inc = fmaf(P.erest[q], (P.xi_u[q] * px + P.xi_v[q] * py) - drf, inc);
        g[q] = g[q] + inc;
    }
    pp_first_moments<MODEL>(P, g, su, sv);
    const float rh = (float)c.rho;
    const FF R{rh, (float)(c.rho - (double)rh)};
    c.U = __fadd_rn(su.hi, su.lo) / rh;
    c.V = __fadd_rn(sv.hi, sv.lo) / rh;
    c.U += P.hDt * fx / rh;
    c.V += P.hDt * fy / rh;
    const FF p = cs_p(P, R);
    cs_psi(P, R, p, c.scg, c.psi, c.psil);
    c.p = ff_to_double(p);
    return c;
}

}  // namespace f32
}  // namespace dugks
