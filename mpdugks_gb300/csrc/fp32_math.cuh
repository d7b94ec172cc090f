// Per-cell arithmetic of the FP32 deviation-storage step, shared by the
// tile kernel (fp32_fused.cu) and the streaming kernel (fp32_stream.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "dugks_device.cuh"
#include "fp32_state.cuh"

namespace dugks {
namespace f32 {

template <typename R>
__device__ __forceinline__ R sxf(int s, R x) { return s > 0 ? x : (s < 0 ? -x : R(0)); }

__device__ __forceinline__ float rsq(float x) { return rsqrtf(x); }

__device__ __forceinline__ double rsq(double x) { return 1.0 / sqrt(x); }
__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// Float-float sum of the nine directions, in a mirror-symmetric tree: the
// pairs of opposite directions first, ((E+W) + (N+S)) + ((NE+SW) + (NW+SE)),
// then the rest direction; a Knuth two-sum at every node and the node errors
// summed in the same tree (depth 4, where a running sum is a chain of 8).
// Returns the head (the rounded tree sum) and, in tail, the summed node errors.
template <typename V, typename Add, typename Sub>
__device__ __forceinline__ V ff_tree9(const V (&a)[9], Add add, Sub sub, V &tail) {
    auto ts = [&](V x, V y, V &e) {
        const V s = add(x, y);
        const V bb = sub(s, x);
        e = add(sub(x, sub(s, bb)), sub(y, bb));
        return s;
    };
    V e15, e37, e26, e48, eA, eB, eC, eD;
    const V s15 = ts(a[1], a[5], e15), s37 = ts(a[3], a[7], e37);
    const V s26 = ts(a[2], a[6], e26), s48 = ts(a[4], a[8], e48);
    const V sA = ts(s15, s37, eA), sB = ts(s26, s48, eB);
    const V sC = ts(sA, sB, eC);
    const V sD = ts(sC, a[0], eD);
    tail = add(add(add(add(e15, e37), eA), add(add(e26, e48), eB)), add(eC, eD));
    return sD;
}
// the same sum as one value (head + tail rounded once)
template <typename V>
__device__ __forceinline__ V ff_sum9(const V (&a)[9]) {
    V tail;
    const V head = ff_tree9(a, [](V x, V y) { return x + y; }, [](V x, V y) { return x - y; }, tail);
    return head + tail;
}
// Macroscopic state of one cell after the update of the previous step
// (Update_MacroVar) from its flow deviations and its phase field phi; HCZ needs
// the previous force and density gradient (aux), AC has u = 0.
template <int MODEL, typename R>
__device__ __forceinline__ void cell_macros(const PR<R> &P, const R *df, R phi, R fx_old, R fy_old, R rx_old,
                                            R ry_old, R &rho, R &U, R &V, R &dp) {
    rho = P.aPhi * phi + P.bPhi;
    if (MODEL == AC) {
        const R fa[9] = {R(0.), df[1], df[2], df[3], df[4], df[5], df[6], df[7], df[8]};
        U = R(0.);
        V = R(0.);
        dp = ff_sum9(fa) * P.Kp;
    } else {
        R ua[9], va[9], fa[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            fa[q] = df[q];
            ua[q] = sxf(d2q9_xu(q), df[q]);
            va[q] = sxf(d2q9_xv(q), df[q]);
        }
        const R su = ff_sum9(ua), sv = ff_sum9(va), sfv = ff_sum9(fa);
        const R inv = R(1.) / (rho * P.RT);
        U = su * inv + P.hDt * fx_old * inv;
        V = sv * inv + P.hDt * fy_old * inv;
        dp = sfv + P.hDt * (rx_old * U + ry_old * V) * P.RT;
    }
}

// MacroSource (Ark/Cpp/SourceM.cpp:35-62) from the 3x3 phi stencil of the cell.
// The stencil's phi values are float-float pairs (x: head, y: tail; the tails are
// zero in FP64) and enter as differences to the centre cell, d = (X - C), each
// formed head with head and tail with tail: a difference of nearby values is then
// correct to the working precision of the difference itself.  Formed from FP32
// values of phi instead, the Laplacian's sum 4 sum(axis) + sum(diag) - 20 phi keeps
// the rounding of numbers near 20 on a result that the bulk term of the chemical
// potential nearly cancels.  ph = {E, W, N, S, NE, NW, SE, SW}.
template <typename R, typename T>
__device__ __forceinline__ void macro_source9(const PR<R> &P, R phi, T C, const T (&ph)[8], R rho, R U, R V, R ppu,
                                              R ppv, R &srcx, R &srcy, R &rhox, R &rhoy, R &fx, R &fy) {
    R d[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) d[k] = (ph[k].x - C.x) + (ph[k].y - C.y);
    const R E = d[0], W = d[1], N = d[2], S = d[3], NE = d[4], NW = d[5], SE = d[6], SW = d[7];
    // mirror-symmetric association: x -> -x maps every sum onto its exact negation
    R gx = (R(4.) * (E - W) + ((NE - NW) + (SE - SW))) * P.inv_12dx;
    R gy = (R(4.) * (N - S) + ((NE - SE) + (NW - SW))) * P.inv_12dy;
    const R lap = (R(4.) * ((E + W) + (N + S)) + ((NE + SW) + (NW + SE))) * P.inv_6dd;
    if (fabs(gx) < R(DUGKS_F32_GCLAMP)) gx = R(0.);
    if (fabs(gy) < R(DUGKS_F32_GCLAMP)) gy = R(0.);
    const R F = R(2.) * P.Beta * (phi - P.PhiL) * (phi - P.PhiV) * (R(2.) * phi - P.PhiL - P.PhiV) - P.Kappa * lap;
    rhox = P.aPhi * gx;
    rhoy = P.aPhi * gy;
    fx = F * gx;
    fy = F * gy;
    if (P.gravity) fy -= P.Gy * (rho - P.RhoL);
    const R L2 = gx * gx + gy * gy;
    const R dU = phi * U - ppu, dV = phi * V - ppv;
    if (L2 != R(0.)) {
        const R tmp = -R(4.) * (phi - P.PhiL) * (phi - P.PhiV) * P.inv_wI_dphi;
        const R k = tmp * rsq(L2);
        srcx = gx * k + dU * P.inv_RTdt;
        srcy = gy * k + dV * P.inv_RTdt;
    } else {
        srcx = dU * P.inv_RTdt;
        srcy = dV * P.inv_RTdt;
    }
}

// ---- packed pairs: every per-direction quantity of the step is carried as the
// pair (flow f_q, phase field h_q); for R = float the pair arithmetic is the
// sm_100+ packed FP32x2 instructions (one issue slot for two lanes' worth).
template <typename R> struct Pair;
template <> struct Pair<float> { using T = float2; };
template <> struct Pair<double> { using T = double2; };

__device__ __forceinline__ float2 mk2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ double2 mk2(double a, double b) { return make_double2(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ double2 add2(double2 a, double2 b) { return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y)); }
__device__ __forceinline__ double2 sub2(double2 a, double2 b) { return make_double2(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y)); }
__device__ __forceinline__ double2 mul2(double2 a, double2 b) { return make_double2(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)); }
__device__ __forceinline__ double2 fma2(double2 a, double2 b, double2 c) {
    return make_double2(__fma_rn(a.x, b.x, c.x), __fma_rn(a.y, b.y, c.y));
}
template <typename T> __device__ __forceinline__ T neg2(T a) { return mk2(-a.x, -a.y); }

template <typename T>
__device__ __forceinline__ T ff_sum9_ht(const T (&a)[9], T &tail) {
    return ff_tree9(a, [](T x, T y) { return add2(x, y); }, [](T x, T y) { return sub2(x, y); }, tail);
}
__device__ __forceinline__ float2 ff_sum9(const float2 (&a)[9]) {
    float2 tail;
    const float2 head = ff_sum9_ht(a, tail);
    return add2(head, tail);
}
__device__ __forceinline__ double2 ff_sum9(const double2 (&a)[9]) {
    double2 tail;
    const double2 head = ff_sum9_ht(a, tail);
    return add2(head, tail);
}

// ---- the phase field phi as a float-float pair (x: head, y: tail; the tail is zero
// in FP64).  Differences of neighbouring values are formed head with head and tail
// with tail, which is exact for the heads of nearby values.
template <typename T>
__device__ __forceinline__ auto pdiff(T a, T b) -> decltype(a.x) {
    return (a.x - b.x) + (a.y - b.y);
}
// phi + d as a pair, d small (Knuth two-sum of the heads, the tails added, renormalised)
template <typename T, typename R>
__device__ __forceinline__ T phi_add(T a, R d) {
    const R s = a.x + d;
    const R bb = s - a.x;
    const R e = (a.x - (s - bb)) + (d - bb);
    const R lo = e + a.y;
    const R hi = s + lo;
    return mk2(hi, lo - (hi - s));
}
// Wall ghost value 2 a - b of two phi pairs (Ark/Cpp/Boundary.cpp:38-63), the head's
// rounding error moved into the tail.
template <typename T>
__device__ __forceinline__ T ghost_pair(T a, T b) {
    const auto two_a = a.x + a.x, nb = -b.x;
    const auto s = two_a + nb;
    const auto bb = s - two_a;
    const auto e = (two_a - (s - bb)) + (nb - bb);
    return mk2(s, e + ((a.y + a.y) - b.y));
}

// mirror-symmetric sum of directions 1..8: ((E+W)+(N+S)) + ((NE+SW)+(NW+SE)), which
// every mirror of the lattice maps onto itself
template <typename T>
__device__ __forceinline__ T sym8p(const T *a) {
    return add2(add2(add2(a[1], a[5]), add2(a[3], a[7])), add2(add2(a[2], a[6]), add2(a[4], a[8])));
}
// Sums over a cell's nine stored deviations (sum f and sum g; the first moments): a plain
// mirror-symmetric sum.  The values are small deviations and remainders; float-float
// sums here changed the errors against FP64 by less than 15 % and cost 8 % of the
// streaming step (4.5 % the zeroth, 3.5 % the first moments).
template <typename T>
__device__ __forceinline__ T dev_sum9(const T (&a)[9]) {
    return add2(a[0], sym8p(a));
}


// 1/x: the hardware approximation refined by one Newton-Raphson step, r' = r + r (1 - x r)
// (the residual by fma): within an ulp, and no special-case branch (x = rho RT here: a
// positive normal number)
__device__ __forceinline__ float rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return fmaf(r, fmaf(-x, r, 1.0f), r);
}
__device__ __forceinline__ double rcp(double x) { return 1.0 / x; }

// direction slots of the faces: the six directions with a non-zero normal velocity
__host__ __device__ constexpr int xslot(int q) { return q == 1 ? 0 : q == 2 ? 1 : q == 4 ? 2 : q == 5 ? 3 : q == 6 ? 4 : q == 8 ? 5 : -1; }
__host__ __device__ constexpr int yslot(int q) { return q == 2 ? 0 : q == 3 ? 1 : q == 4 ? 2 : q == 6 ? 3 : q == 7 ? 4 : q == 8 ? 5 : -1; }

// asynchronous 4- or 8-byte global -> shared copies (cp.async)
template <typename R>
__device__ __forceinline__ void cp_async(R *smem, const R *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    if (sizeof(R) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Site terms of the equilibria and force sources (a cell or a face), shared by
// all directions: u/RT, |u|^2 lambda, rho RT, u.F, u.grad rho, and the pairs
// (rho RT, phi), (dp, dphi) of the packed equilibria.
template <typename R>
struct EqSite {
    typename Pair<R>::T A2, D2;
    R Ux, Vx, uuL, UF, UR, fx, fy, rx, ry, sx, sy, fxI, fyI, dpI;
};
template <int MODEL, typename R>
__device__ __forceinline__ EqSite<R> eq_site(const PR<R> &P, R U, R V, R uu, R rho, R phi, R dp, R dphi, R fx,
                                              R fy, R rx, R ry, R sx_, R sy_) {
    EqSite<R> e;
    e.fx = fx;
    e.fy = fy;
    e.sx = sx_;
    e.sy = sy_;
    if (MODEL == AC) {
        e.fxI = fx * P.invRT;
        e.fyI = fy * P.invRT;
        e.dpI = dp * P.invRT;
        e.D2 = mk2(e.dpI, dphi);
    } else {
        e.Ux = U * P.invRT;
        e.Vx = V * P.invRT;
        e.uuL = uu * P.Lambda0;
        e.UF = U * fx + V * fy;
        e.UR = U * rx + V * ry;
        e.rx = rx;
        e.ry = ry;
        e.A2 = mk2(rho * P.RT, phi);
        e.D2 = mk2(dp, dphi);
    }
    return e;
}

// Equilibrium deviations and force terms, as (f, h) pairs, of direction Q in
// {1, 2, 3, 4} and of its opposite Q+4, which share every term up to a sign:
//   Eq = w (dp + rho RT G, dphi + u1 phi) (HCZ) or w (dp/RT, dphi) (AC),
//   So = (w (A + G (A + RT B)), w xi.src) with A = xi.F - u.F, B = xi.grad rho -
//   u.grad rho, G = u1 + u1^2/2 - |u|^2 lambda (= (1+G)(c.F) + G RT (c.grad rho),
//   c = xi - u), u1 = xi.u / RT.
template <int MODEL, int Q, typename R>
__device__ __forceinline__ void eq_pair(const PR<R> &P, const EqSite<R> &e, typename Pair<R>::T &Eq,
                                        typename Pair<R>::T &So, typename Pair<R>::T &Eqb,
                                        typename Pair<R>::T &Sob) {
    constexpr int xu = d2q9_xu(Q), xv = d2q9_xv(Q);
    const R wq = (R)d2q9_w(Q);
    const R hS = wq * (sxf(xu, e.sx) + sxf(xv, e.sy));
    if (MODEL == AC) {
        Eq = mul2(mk2(wq, wq), e.D2);
        Eqb = Eq;
        const R sf = wq * (sxf(xu, e.fxI) + sxf(xv, e.fyI));
        So = mk2(sf, hS);
        Sob = mk2(-sf, -hS);
    } else {
        const R u1 = sxf(xu, e.Ux) + sxf(xv, e.Vx);
        const R H = (R(0.5) * u1) * u1 - e.uuL;
        const R G = H + u1, Gb = H - u1;
        const R eF = sxf(xu, e.fx) + sxf(xv, e.fy), eR = sxf(xu, e.rx) + sxf(xv, e.ry);
        const R A = eF - e.UF, Ab = -eF - e.UF;
        const R B = eR - e.UR, Bb = -eR - e.UR;
        const R C = P.RT * B + A, Cb = P.RT * Bb + Ab;
        const auto w2 = mk2(wq, wq);
        Eq = mul2(w2, fma2(e.A2, mk2(G, u1), e.D2));
        Eqb = mul2(w2, fma2(e.A2, mk2(Gb, -u1), e.D2));
        So = mk2(wq * (G * C + A), hS);
        Sob = mk2(wq * (Gb * Cb + Ab), -hS);
    }
}

// ---- the three per-cell stages of one step, shared by the tile kernel and
// the streaming kernel (same operations in the same order in both)

// Stage 1 of one cell: macroscopic state (from the deviations, or on the first
// step after an initialisation from the state it left), MacroSource on the 3x3
// stencil of phi pairs, centre pc and ph = {E, W, N, S, NE, NW, SE, SW}, and the
// collision increment inc = B - T of every direction.  Pq and inc are (f, h) pairs
// whose h part is relative to w_q phi of this cell: Pq[q].y = g_q, and the h
// equilibrium enters as h_eq - w_q phi = w_q phi u1.  src = {srcx, srcy, rhox, rhoy,
// fx, fy}; phi_o, U_o, V_o for the caller's outputs.  EQOUT: also the equilibria,
// sources and macroscopic state the NEE wall faces need, into *eo.
template <typename R>
struct CellEq {
    typename Pair<R>::T Eq[9], So[9];
    R phi, dp, srcy, tau;
};
template <int MODEL, typename R, bool EQOUT = false>
__device__ __forceinline__ void collide_cell(const PR<R> &P, const SR<R> &S, long long c, int first,
                                             const typename Pair<R>::T (&Pq)[9], R sfz, const R (&a6)[A_N],
                                             typename Pair<R>::T pc, const typename Pair<R>::T (&ph)[8],
                                             typename Pair<R>::T (&inc)[9], R (&src)[6], R &phi_o, R &U_o, R &V_o,
                                             CellEq<R> *eo = nullptr) {
    using T = typename Pair<R>::T;
    R phi = pc.x + pc.y, rho = R(0.), U = R(0.), V = R(0.), dp = R(0.);
    R srcx = R(0.), srcy = R(0.), rhox = R(0.), rhoy = R(0.), fx = R(0.), fy = R(0.);
    R aBP, cBP, rxo = R(0.), ryo = R(0.), tau_c = P.tauf;
    if (first) {
        // first step after an initialisation: the reference uses the state the
        // initialisation left (p0, zero forces, tau from Mu0), as uploaded
        const R *I = S.init;
        const long long ps = (long long)S.qs;
        rho = I[I_RHO * ps + c];
        U = I[I_U * ps + c];
        V = I[I_V * ps + c];
        dp = I[I_DP * ps + c];
        srcx = I[I_SRCX * ps + c];
        srcy = I[I_SRCY * ps + c];
        rhox = I[I_RHOX * ps + c];
        rhoy = I[I_RHOY * ps + c];
        fx = I[I_FX * ps + c];
        fy = I[I_FY * ps + c];
        const R tau = I[I_TAU * ps + c];
        tau_c = tau;
        aBP = (R(2.) * tau - P.hDt) / (R(2.) * tau + P.dt);
        cBP = tau * (R(1.) - aBP);
    } else {
        rho = P.aPhi * phi + P.bPhi;
        R ppu = R(0.), ppv = R(0.);
        if (MODEL == AC) {
            dp = sfz * P.Kp;
        } else {
            const R fxo = a6[A_FX], fyo = a6[A_FY];
            rxo = a6[A_RHOX];
            ryo = a6[A_RHOY];
            ppu = a6[A_PPU];
            ppv = a6[A_PPV];
            // first moments (sum xi_x f, sum xi_y f)
            const T mt[9] = {mk2(R(0.), R(0.)),     mk2(Pq[1].x, R(0.)),    mk2(Pq[2].x, Pq[2].x),
                             mk2(R(0.), Pq[3].x),   mk2(-Pq[4].x, Pq[4].x), mk2(-Pq[5].x, R(0.)),
                             mk2(-Pq[6].x, -Pq[6].x), mk2(R(0.), -Pq[7].x), mk2(Pq[8].x, -Pq[8].x)};
            const T mv = dev_sum9(mt);
            const R inv = rcp(rho * P.RT);
            U = mv.x * inv + P.hDt * fxo * inv;
            V = mv.y * inv + P.hDt * fyo * inv;
            dp = sfz + P.hDt * (rxo * U + ryo * V) * P.RT;
        }
        macro_source9(P, phi, pc, ph, rho, U, V, ppu, ppv, srcx, srcy, rhox, rhoy, fx, fy);
        aBP = P.aBP_f;  // tau is constant after the first step (nu_L = nu_V)
        cBP = P.tauf * (R(1.) - aBP);
    }
    const R bBP = R(1.) - aBP;
    const R uu = U * U + V * V;
    // equilibria of q != 0; q = 0 from the exact zeroth moment (sum dEq = dp for
    // HCZ, 0 for AC; sum (h_eq - w phi) = 0), so FP32 weights cannot leak mass
    T Eq[9], So[9];
    const EqSite<R> es = eq_site<MODEL, R>(P, U, V, uu, rho, phi, dp, R(0.), fx, fy, rhox, rhoy, srcx, srcy);
    eq_pair<MODEL, 1>(P, es, Eq[1], So[1], Eq[5], So[5]);
    eq_pair<MODEL, 2>(P, es, Eq[2], So[2], Eq[6], So[6]);
    eq_pair<MODEL, 3>(P, es, Eq[3], So[3], Eq[7], So[7]);
    eq_pair<MODEL, 4>(P, es, Eq[4], So[4], Eq[8], So[8]);
    const T sEq = sym8p(Eq);
    Eq[0] = sub2(mk2(MODEL == AC ? R(0.) : dp, R(0.)), sEq);
    if (MODEL == AC) {
        So[0] = mk2(R(0.), R(0.));
    } else {
        const R G0 = -uu * P.Lambda0;
        const R wq = (R)d2q9_w(0);
        So[0] = mk2(wq * ((R(1.) + G0) * (-U * fx - V * fy) + G0 * P.RT * (-U * rhox - V * rhoy)), R(0.));
    }
    // collision increment B - T = (1-a)(Eq - T) + c S: small near equilibrium,
    // so B = T + increment keeps the rest state and rounds relative to the increment
    const T b2 = mk2(bBP, P.h_bBP), c2 = mk2(cBP, P.h_cBP);
#pragma unroll
    for (int q = 0; q < 9; ++q) inc[q] = fma2(b2, sub2(Eq[q], Pq[q]), mul2(c2, So[q]));
    // the rest directions take the exact zeroth moments of the collision:
    // phase field sum_q h is conserved (sum Eq = phi, sum S = 0); HCZ flow
    //   (1-a)(p - sum f) + c sum S = (1-a) hDt RT (grad rho_old . u) + c RT (u . grad rho)
    const T sInc = sym8p(inc);
    const R z0 = MODEL == HCZ ? (bBP * P.hDt * P.RT * (rxo * U + ryo * V) + cBP * P.RT * (U * rhox + V * rhoy)) - sInc.x
                              : inc[0].x;
    inc[0] = mk2(z0, -sInc.y);
    src[0] = srcx;
    src[1] = srcy;
    src[2] = rhox;
    src[3] = rhoy;
    src[4] = fx;
    src[5] = fy;
    phi_o = phi;
    U_o = U;
    V_o = V;
    if (EQOUT) {
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            eo->Eq[q] = Eq[q];
            eo->So[q] = So[q];
        }
        eo->phi = phi;
        eo->dp = dp;
        eo->srcy = srcy;
        eo->tau = tau_c;
    }
}

// NEE wall face (Wall_3_NEE, Ark/Cpp/Boundary.cpp:140-184, then Wall_3_BB) of a wall row's
// cell from its collision state ce and stored deviations Pq: the equilibrium at the wall
// (the face velocity stays 0, phi extrapolated to the face with the MacroSource vector,
// Phi_y, the reference's choice) plus the cell's non-equilibrium part f - Eq + hDt S times
// 2 tau / (2 tau + dt) (h: 2 TauMass / (2 TauMass + dt)), the directions entering the fluid
// bounced back; fluxes xi.n of the six directions crossing the face, the f parts as
// deviations and the h parts relative to w_q avg (the face phi the update's flux
// divergence takes for it).  side: 0 the bottom wall (below the cell), 1 the top.
template <int MODEL, typename R>
__device__ __forceinline__ void nee_wall_flux(const PR<R> &P, const CellEq<R> &ce,
                                              const typename Pair<R>::T (&Pq)[9], R avg, int side,
                                              typename Pair<R>::T (&F)[6]) {
    using T = typename Pair<R>::T;
    const R dyw = side ? R(0.5) : R(-0.5);
    const R Phi_w = ce.phi + ce.srcy * dyw;
    const R fneq = R(2.) * ce.tau / (R(2.) * ce.tau + P.dt);
    T v[9];
#pragma unroll
    for (int q = 1; q < 9; ++q) {
        const R wq = (R)d2q9_w(q);
        // the wall equilibrium at u = 0 as a deviation: w (p - p0) (HCZ), w (p - p0) / RT (AC)
        const R feq = MODEL == AC ? wq * ce.dp * P.invRT : wq * ce.dp;
        const T ne = fma2(mk2(P.hDt, P.hDt), ce.So[q], sub2(Pq[q], ce.Eq[q]));
        v[q] = mk2(fma(fneq, ne.x, feq), fma(P.hneq, ne.y, wq * (Phi_w - avg)));
    }
#pragma unroll
    for (int q = 1; q < 9; ++q) {
        const int xv = d2q9_xv(q);
        if (side ? xv < 0 : xv > 0) v[q] = v[d2q9_bb(q)];
    }
#pragma unroll
    for (int q = 1; q < 9; ++q)
        if (d2q9_xv(q) != 0) F[yslot(q)] = d2q9_xv(q) > 0 ? v[q] : neg2(v[q]);
}

// Phase-field inputs of one face: avg = (phi_o + phi_n)/2 (the face's h reference is
// w_q avg), dn = phi_n - phi_o, dt = the tangential difference of phi summed over the
// two cells (the same combination D(q) forms of the f-bar-plus values), all from pairs.
template <typename R>
struct FacePhi {
    R avg, dn, dt;
};
// x-face between o (west) and n (east); u / d: the cells above / below each
template <typename T>
__device__ __forceinline__ FacePhi<decltype(T::x)> face_phi_x(T o, T n, T nu, T nd, T ou, T od) {
    using R = decltype(T::x);
    return {R(0.5) * (o.x + n.x), pdiff(n, o), pdiff(nu, nd) + pdiff(ou, od)};
}
// y-face between o (below) and n (above); w / e: the cells west / east of each
template <typename T>
__device__ __forceinline__ FacePhi<decltype(T::x)> face_phi_y(T o, T n, T nw, T ne, T ow, T oe) {
    using R = decltype(T::x);
    return {R(0.5) * (o.x + n.x), pdiff(n, o), pdiff(nw, ne) + pdiff(ow, oe)};
}

template <int MODEL, bool XF, typename R>
__device__ __forceinline__ void face_state_flux(const PR<R> &P, const typename Pair<R>::T (&bh)[9], const R (&av)[6],
                                                R avg, int wall, typename Pair<R>::T (&F)[6]);

// Stage 2 of one face: half-step reconstruction at the face midpoint, face
// moments, equilibria of the six directions crossing the face and their
// fluxes xi.n (f, h pairs, slot order xslot / yslot).  XF: an x-face (normal
// +x) between o = (r, e-1) and n = (r, e), else a y-face between o = (r-1, e)
// and n = (r, e).  Accessors: O(q), N(q) the f-bar-plus pairs of the two cells;
// D(q) the tangential central difference summed over the two cells
// ((n+t) - (n-t)) + ((o+t) - (o-t)) with t the tangential neighbour offset
// (x-face: +y; y-face: -x); av = face averages of {srcx, srcy, rhox, rhoy, fx,
// fy}; wall: 0, or 1 / 2 for the bottom / top wall face (bounce-back).
// The h parts are relative to w_q phi of their cell; the face works relative to
// w_q fp.avg: the reconstruction of w_q phi adds w_q (L_q(phi) - avg) from fp, and
// the fluxes F[q].y returned are those of h_q - w_q fp.avg (the w_q avg parts of a
// cell's four faces are added by the update from the phi differences).
template <int MODEL, bool XF, typename R, typename FO, typename FN, typename FD>
__device__ __forceinline__ void face_flux(const PR<R> &P, FO &&O, FN &&N, FD &&D, const R (&av)[6],
                                          const FacePhi<R> &fp, int wall, typename Pair<R>::T (&F)[6]) {
    using T = typename Pair<R>::T;
    const T half = mk2(R(0.5), R(0.5));
    T bh[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const int xu = d2q9_xu(q), xv = d2q9_xv(q);
        const T o = O(q), n = N(q);
        const T avg = mul2(half, add2(o, n));
        const int sn = XF ? xu : xv, st = XF ? xv : xu;  // normal / tangential velocity
        if (sn == 0 && st == 0) {
            bh[q] = avg;
            continue;
        }
        // avg - hDt xi.grad: the normal part (o - n)/(-d) is folded into the two
        // cells' weights 1/2 -+ hDt sn/(-d) (0.25 and 0.75 on unit cells, exact),
        // the tangential central difference, averaged over the two cells of the
        // face, enters with the weight -hDt st/(4 d_t); the phase field's w_q phi
        // part takes the same weights on phi: w_q (cn (phi_n - phi_o) + k dt)
        T b = avg;
        R wphi = R(0.);
        if (sn != 0) {
            const R rn = XF ? P.r_ndx : P.r_ndy;
            const R cn = P.hDt * ((R)sn * rn);
            b = fma2(n, mk2(R(0.5) + cn, R(0.5) + cn), mul2(o, mk2(R(0.5) - cn, R(0.5) - cn)));
            wphi = cn * fp.dn;
        }
        if (st != 0) {
            const T d = D(q);
            const R rt = XF ? P.r_2dy : P.r_n2dx;
            const R k = -(P.hDt * (R(0.5) * (R)st * rt));
            b = fma2(d, mk2(k, k), b);
            wphi = fma(k, fp.dt, wphi);
        }
        b.y = fma((R)d2q9_w(q), wphi, b.y);
        bh[q] = b;
    }
    face_state_flux<MODEL, XF, R>(P, bh, av, fp.avg, wall, F);
}

// The rest of a face from its reconstructed half-step state bh (f deviations, h relative
// to w_q avg, avg the face's phi reference): face moments, equilibria of the six
// directions crossing the face, bounce-back at a wall face, fluxes xi.n (slot order
// xslot / yslot).  Shared by the central (face_flux) and upwind reconstructions.
template <int MODEL, bool XF, typename R>
__device__ __forceinline__ void face_state_flux(const PR<R> &P, const typename Pair<R>::T (&bh)[9], const R (&av)[6],
                                                R avg, int wall, typename Pair<R>::T (&F)[6]) {
    using T = typename Pair<R>::T;
    // face moments (sum f, sum h) with the mirror-symmetric association
    const T z = add2(mk2(MODEL == AC ? R(0.) : bh[0].x, bh[0].y), sym8p(bh));
    // dphif: the face phi relative to fp.avg
    const R sf = z.x, dphif = z.y;
    const R su = (bh[1].x - bh[5].x) + ((bh[2].x - bh[6].x) + (bh[8].x - bh[4].x));
    const R sv = (bh[3].x - bh[7].x) + ((bh[2].x - bh[6].x) + (bh[4].x - bh[8].x));
    const R phif = avg + dphif;
    const R rhof = P.aPhi * phif + P.bPhi;
    R Uf, Vf, dpf;
    if (MODEL == AC) {
        Uf = R(0.);
        Vf = R(0.);
        dpf = sf * P.Kp;
    } else {
        const R inv = rcp(rhof * P.RT);
        Uf = su * inv + R(0.5) * P.hDt * av[4] * inv;
        Vf = sv * inv + R(0.5) * P.hDt * av[5] * inv;
        dpf = sf + R(0.5) * P.hDt * P.RT * (av[2] * Uf + av[3] * Vf);
    }
    const R uu = Uf * Uf + Vf * Vf;
    const T a2 = mk2(P.ah_f, P.h_ah), c2 = mk2(P.tauf * (R(1.) - P.ah_f), P.h_ch);
    // face distributions of the six directions crossing the face (three opposite
    // pairs): Eq + a (bh - Eq) + c S
    T out[9];
    const EqSite<R> es = eq_site<MODEL, R>(P, Uf, Vf, uu, rhof, phif, dpf, dphif, av[4], av[5], av[2], av[3], av[0],
                                           av[1]);
    auto face_pair = [&](auto QC) {
        constexpr int Qa = decltype(QC)::value, Qb = Qa + 4;
        T Eq, So, Eqb, Sob;
        eq_pair<MODEL, Qa>(P, es, Eq, So, Eqb, Sob);
        out[Qa] = fma2(c2, So, fma2(a2, sub2(bh[Qa], Eq), Eq));
        out[Qb] = fma2(c2, Sob, fma2(a2, sub2(bh[Qb], Eqb), Eqb));
    };
    if (XF) face_pair(std::integral_constant<int, 1>());  // E, W
    else face_pair(std::integral_constant<int, 3>());     // N, S
    face_pair(std::integral_constant<int, 2>());          // NE, SW
    face_pair(std::integral_constant<int, 4>());          // NW, SE
    if (!XF && wall) {
        // bounce-back of the directions entering the fluid (Ark/Cpp/Boundary.cpp:118-139)
        const bool bottom = wall == 1;
#pragma unroll
        for (int q = 1; q < 9; ++q) {
            const int xv = d2q9_xv(q);
            if (xv != 0 && (bottom ? xv > 0 : xv < 0)) out[q] = out[d2q9_bb(q)];
        }
    }
    // fluxes xi.n (f, h) of the six directions
#pragma unroll
    for (int q = 1; q < 9; ++q) {
        if (XF && d2q9_xu(q) != 0) F[xslot(q)] = d2q9_xu(q) > 0 ? out[q] : neg2(out[q]);
        if (!XF && d2q9_xv(q) != 0) F[yslot(q)] = d2q9_xv(q) > 0 ? out[q] : neg2(out[q]);
    }
}

// Stage 3 of one cell: the finite-volume update (Update_phi_T) of the
// deviations, 4/3 B - 1/3 T = T + (4/3)(B - T) + dt/V sum(F), as the old value plus
// one small increment rounded to nearest into storage (the stored values are small:
// a stochastic rounding gave the same errors against FP64 over 10000 steps, and its
// random bits cost ~10 % of the step).  The h parts: the
// face fluxes carry h_q - w_q avg(phi) of their face, so
//   phi_new = phi + dphi,  dphi = dt/V sum_q (sum of the cell's h fluxes of q)
// (the w_q avg(phi) parts cancel: sum_q w_q xi_q = 0, and sum_q (B - T) = 0), and
//   g_q,new = g_q + (4/3) inc_q + dt/V (h flux sum of q)
//             + w_q (xi_q,x px + xi_q,y py) - w_q dphi   (q = 1..8),
// px = dt/V (phi_W - phi_E)/2, py = dt/V (phi_S - phi_N)/2: the w_q avg(phi) flux
// divergence on unit cells.  dn[q].y (q >= 1) is g_q,new; dn[0].y is not used.
template <typename R>
__device__ __forceinline__ void update_cell(const PR<R> &P, const typename Pair<R>::T (&Pq)[9],
                                            const typename Pair<R>::T (&inc)[9], const typename Pair<R>::T (&FW)[6],
                                            const typename Pair<R>::T (&FE)[6], const typename Pair<R>::T (&FS)[6],
                                            const typename Pair<R>::T (&FN)[6], R px, R py,
                                            typename Pair<R>::T (&dn)[9], R &dphi) {
    using T = typename Pair<R>::T;
    const T btp = mk2(P.bTP, P.bTP), dtv = mk2(P.dtV, P.dtV);
    T s[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        // net flux (W - E) + (S - N) with the mirror-symmetric association
        s[q] = mk2(R(0.), R(0.));
        const int xs = xslot(q), ys = yslot(q);
        if (xs >= 0 && ys >= 0) s[q] = add2(sub2(FW[xs], FE[xs]), sub2(FS[ys], FN[ys]));
        else if (xs >= 0) s[q] = sub2(FW[xs], FE[xs]);
        else if (ys >= 0) s[q] = sub2(FS[ys], FN[ys]);
    }
    dphi = P.dtV * sym8p(s).y;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const int xs = xslot(q), ys = yslot(q);
        // old value plus one small increment
        T incr = (xs >= 0 || ys >= 0) ? fma2(dtv, s[q], fma2(btp, inc[q], inc[q])) : fma2(btp, inc[q], inc[q]);
        if (q > 0) {
            const R wq = (R)d2q9_w(q);
            incr.y = fma(wq, (sxf(d2q9_xu(q), px) + sxf(d2q9_xv(q), py)) - dphi, incr.y);
        }
        dn[q] = add2(Pq[q], incr);
    }
}


}  // namespace f32
}  // namespace dugks
