// FP32 deviation-storage DUGKS step: one fused kernel per time step.
//
// Storage: f~ and h~ as FP32 deviations from fixed rest equilibria,
//   HCZ: f0_q = w_q p0;  AC: f0_q = w_q p0/RT - [q=0] p0/RT;  h0_q = w_q phi0,
// (p0 = 1, phi0 = 1/2).  Every step relation of the reference is affine with
// coefficients that sum to one (aBP + bBP = 1, ah + bh = 1, 4/3 - 1/3 = 1)
// and the rest parts of the four face fluxes of a cell cancel (sum of
// +-xi.n = 0, bounce-back maps q to a direction of equal weight), so the step
// is carried out on the deviations directly; the rest moments enter only the
// macroscopic quantities (p = p0 + dp, phi = phi0 + dphi).  Cell moment sums
// (phi, rho u, rho v, p) are float-float (Knuth two-sum) sums of the FP32
// deviations; the domain sums and residual are FP64 reductions.
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
//
// Phase references: P1 Ark/Cpp/DUGKS2DSolver.cpp:175-183 (Ark/Lib/D2Q9HCZ.cpp:54-92,
// Ark/Lib/D2Q9AC.cpp:69-105); P4 :219-250 (CD_Interior_phi_Bh :604-687);
// P8 :748-792; P9 Ark/Lib/D2Q9HCZ.cpp:133-182; P10 Ark/Cpp/SourceM.cpp:35-62.
#include <cuda_runtime.h>

#include <cstdint>

#include "dugks_device.cuh"
#include "fp32_state.cuh"

namespace dugks {
namespace f32 {

constexpr int TW = 30, TH = 14;  // interior tile
constexpr int BX = 32, BY = 16;  // threads = tile + halo ring

// Knuth two-sum accumulation (float-float for R = float)
template <typename R>
struct FFs {
    R hi = 0, lo = 0;
    __device__ __forceinline__ void add(R b) {
        const R s = hi + b;
        const R bb = s - hi;
        const R err = (hi - (s - bb)) + (b - bb);
        hi = s;
        lo += err;
    }
    __device__ __forceinline__ R value() const { return hi + lo; }
};

template <typename R>
__device__ __forceinline__ R sxf(int s, R x) { return s > 0 ? x : (s < 0 ? -x : R(0)); }

// sum of directions 1..8 (E,NE,N,NW,W,SW,S,SE) in an order that every mirror of
// the lattice maps onto itself: ((E+W)+(N+S)) + ((NE+SW)+(NW+SE))
template <typename R>
__device__ __forceinline__ R sym8(const R *a) {
    return ((a[1] + a[5]) + (a[3] + a[7])) + ((a[2] + a[6]) + (a[4] + a[8]));
}
__device__ __forceinline__ float rsq(float x) { return rsqrtf(x); }

// Stochastic rounding of a + b to the storage type.  The exact sum is
// s + err (two-sum); s is moved to its neighbour toward err with probability
// |err| / ulp.  Without it, a state that is nearly steady repeats the same
// FP32 rounding every step and the error grows linearly with the step count;
// with it the rounding errors are unbiased and uncorrelated (random-walk
// growth).  key: a per (cell, velocity, step) counter hashed to 24 bits.
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float add_sr(float a, float b, uint32_t key) {
    const float s = a + b;
#if defined(DUGKS_F32_NO_SR)
    return s;
#endif
    const float bb = s - a;
    const float err = (a - (s - bb)) + (b - bb);
    if (err == 0.f) return s;
    const float nb = nextafterf(s, err > 0.f ? INFINITY : -INFINITY);
    const float ulp = fabsf(nb - s);
    const float u = (float)(mix32(key) >> 8) * (1.0f / 16777216.0f);
    return (u * ulp < fabsf(err)) ? nb : s;
}
__device__ __forceinline__ double add_sr(double a, double b, uint32_t) { return a + b; }
__device__ __forceinline__ double rsq(double x) { return 1.0 / sqrt(x); }
__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// Macroscopic state of one cell after the update of the previous step
// (Update_MacroVar), from its deviations; HCZ needs the previous force and
// density gradient (aux), AC has u = 0.
template <int MODEL, typename R>
__device__ __forceinline__ void cell_macros(const PR<R> &P, const R *df, const R *dh, R fx_old,
                                            R fy_old, R rx_old, R ry_old, R &dphi, R &rho,
                                            R &U, R &V, R &dp) {
    FFs<R> sh, sf, su, sv;
#pragma unroll
    for (int q = 0; q < 9; ++q) sh.add(dh[q]);  // two-sum: exact to 2^-48, order-independent after rounding
    dphi = sh.value();
    const R phi = P.phi0 + dphi;
    rho = P.aPhi * phi + P.bPhi;
    if (MODEL == AC) {
#pragma unroll
        for (int q = 1; q < 9; ++q) sf.add(df[q]);
        U = R(0.);
        V = R(0.);
        dp = sf.value() * P.Kp;
    } else {
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            sf.add(df[q]);
            if (d2q9_xu(q)) su.add(sxf(d2q9_xu(q), df[q]));
            if (d2q9_xv(q)) sv.add(sxf(d2q9_xv(q), df[q]));
        }
        const R inv = R(1.) / (rho * P.RT);
        U = su.value() * inv + P.hDt * fx_old * inv;
        V = sv.value() * inv + P.hDt * fy_old * inv;
        dp = sf.value() + P.hDt * (rx_old * U + ry_old * V) * P.RT;
    }
}

// MacroSource (Ark/Cpp/SourceM.cpp:35-62) on the shared phi tile.
template <typename R>
__device__ __forceinline__ void macro_source32(const PR<R> &P, const R (*sphi)[BX + 2], int r, int e, R phi,
                                               R rho, R U, R V, R ppu, R ppv, R &srcx,
                                               R &srcy, R &rhox, R &rhoy, R &fx, R &fy) {
    // sphi[r+1][e+1] is this cell
    const R E = sphi[r + 1][e + 2], W = sphi[r + 1][e], N = sphi[r + 2][e + 1], S = sphi[r][e + 1];
    const R NE = sphi[r + 2][e + 2], NW = sphi[r + 2][e], SE = sphi[r][e + 2], SW = sphi[r][e];
    // mirror-symmetric association: x -> -x maps every sum onto its exact negation
    R gx = (R(4.) * (E - W) + ((NE - NW) + (SE - SW))) * P.inv_12dx;
    R gy = (R(4.) * (N - S) + ((NE - SE) + (NW - SW))) * P.inv_12dy;
    const R lap = (R(4.) * ((E + W) + (N + S)) + ((NE + SW) + (NW + SE)) - R(20.) * phi) * P.inv_6dd;
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

constexpr size_t SMEM_ELEMS = (size_t)(BY + 2) * (BX + 2) + (18 + 6 + 18) * BY * BX;

template <int MODEL, bool WALLS, typename R>
__global__ void __launch_bounds__(BX *BY, 1) k_step32(PR<R> P, SR<R> S, int first, int gin, int gout,
                                                      uint32_t step) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *smem = reinterpret_cast<R *>(smem_raw);
    R(*sphi)[BX + 2] = reinterpret_cast<R(*)[BX + 2]>(smem);                             // phi, halo 2
    R(*sB)[BY][BX] = reinterpret_cast<R(*)[BY][BX]>(smem + (BY + 2) * (BX + 2));        // f-bar-plus (f 0..8, h 9..17)
    R(*sA)[BY][BX] = sB + 18;                                                             // srcx srcy rhox rhoy fx fy
    R(*sFS)[BY][BX] = sA + 6;                                                             // south-face fluxes
    const int e = threadIdx.x, r = threadIdx.y;
    const int tid = r * BX + e;
    const int nx = P.nx, ny = P.ny, pitch = P.pitch;
    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
    const int w = min(TW, nx - x0), hh = min(TH, ny - y0);
    // extended cell of this thread
    const bool act = (e <= w + 1) && (r <= hh + 1);
    int gi = wrapi(x0 + e - 1, nx);
    int gj = y0 + r - 1;
    bool ghost = false;  // wall ghost row (values extrapolated in shared memory)
    if (WALLS) {
        if (gj < 0 || gj >= ny) ghost = true;
    } else {
        gj = wrapi(gj, ny);
    }
    const bool real = act && !ghost;
    const size_t c = real ? (size_t)gj * pitch + gi : 0;

    // ---- stage 0: own deviations, phi of the halo-2 region
    R df[9], dh[9];
    R dphi = R(0.);
    if (real) {
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            df[q] = S.df[(size_t)q * S.qs + c];
            dh[q] = S.dh[(size_t)q * S.qs + c];
        }
        FFs<R> sh;
#pragma unroll
        for (int q = 0; q < 9; ++q) sh.add(dh[q]);
        dphi = sh.value();
        sphi[r + 1][e + 1] = P.phi0 + dphi;
    } else if (act && WALLS) {
        // ghost phi: the previous step's extrapolation (Ark/Cpp/Boundary.cpp:38-63)
        sphi[r + 1][e + 1] = S.gphi[(size_t)(gin * 2 + (gj < 0 ? 0 : 1)) * pitch + gi];
    }
    {   // ring of the phi region: e in {-1, w+2} or r in {-1, hh+2}
        const int RW = w + 4, RH = hh + 4;  // ring spans e in [-1, w+2], r in [-1, hh+2]
        const int nring = 2 * RW + 2 * (RH - 2);
        for (int k = tid; k < nring; k += BX * BY) {
            int re, rr;
            if (k < RW) { re = k - 1; rr = -1; }
            else if (k < 2 * RW) { re = k - RW - 1; rr = hh + 2; }
            else if (k < 2 * RW + (RH - 2)) { re = -1; rr = k - 2 * RW; }
            else { re = w + 2; rr = k - 2 * RW - (RH - 2); }
            const int ri = wrapi(x0 + re - 1, nx);
            int rj = y0 + rr - 1;
            R v = R(0.);
            if (WALLS && (rj < -1 || rj > ny)) {
                v = R(0.);  // never read: no real cell of this tile reaches it
            } else if (WALLS && (rj == -1 || rj == ny)) {
                v = S.gphi[(size_t)(gin * 2 + (rj < 0 ? 0 : 1)) * pitch + ri];
            } else {
                if (!WALLS) rj = wrapi(rj, ny);
                const size_t cc = (size_t)rj * pitch + ri;
                FFs<R> sh;
#pragma unroll
                for (int q = 0; q < 9; ++q) sh.add(S.dh[(size_t)q * S.qs + cc]);
                v = P.phi0 + sh.value();
            }
            sphi[rr + 1][re + 1] = v;
        }
    }
    __syncthreads();

    // ---- stage 1: macros, MacroSource, f-bar-plus of every real cell of the region
    R phi = P.phi0 + dphi, rho = R(0.), U = R(0.), V = R(0.), dp = R(0.);
    R srcx = R(0.), srcy = R(0.), rhox = R(0.), rhoy = R(0.), fx = R(0.), fy = R(0.);
    R aBP = R(0.), bBP = R(0.), cBP = R(0.);
    R rxo_c = R(0.), ryo_c = R(0.);  // previous density gradient (HCZ pressure)
    R inc[18];  // collision increments B - T of this cell
    if (real) {
        if (first) {
            // first step after an initialisation: the reference uses the state the
            // initialisation left (p0, zero forces, tau from Mu0), as uploaded
            const R *I = S.init;
            const size_t ps = S.qs;
            phi = P.phi0 + I[I_DPHI * ps + c];
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
            aBP = (R(2.) * tau - P.hDt) / (R(2.) * tau + P.dt);
        } else {
            R fxo = R(0.), fyo = R(0.), rxo = R(0.), ryo = R(0.), ppu = R(0.), ppv = R(0.);
            if (MODEL != AC) {
                fxo = S.aux[A_FX * S.qs + c];
                fyo = S.aux[A_FY * S.qs + c];
                rxo = S.aux[A_RHOX * S.qs + c];
                ryo = S.aux[A_RHOY * S.qs + c];
                ppu = S.aux[A_PPU * S.qs + c];
                ppv = S.aux[A_PPV * S.qs + c];
            }
            R d;
            cell_macros<MODEL>(P, df, dh, fxo, fyo, rxo, ryo, d, rho, U, V, dp);
            rxo_c = rxo;
            ryo_c = ryo;
            macro_source32(P, sphi, r, e, phi, rho, U, V, ppu, ppv, srcx, srcy, rhox, rhoy, fx, fy);
            aBP = P.aBP_f;  // tau is constant after the first step (nu_L = nu_V)
        }
        bBP = R(1.) - aBP;
        // f-bar-plus deviations
        const R uu = U * U + V * V;
        // dphi itself, not (phi0 + dphi) - phi0: one rounding less in the zeroth moment
        const R dphi_c = first ? phi - P.phi0 : dphi;
        if (first) {
            // tau = Mu0 / (rho RT) of the initialisation
            const R tau = S.init[I_TAU * S.qs + c];
            cBP = tau * bBP;
        } else {
            cBP = P.tauf * bBP;
        }
        // equilibria of q != 0; q = 0 from the exact zeroth moment (sum dEq = dp for
        // HCZ, 0 for AC; sum dhEq = dphi), so FP32 weights cannot leak mass
        R dEqv[9], fSov[9], dhEqv[9];
        R sEq, shEq;
#pragma unroll
        for (int q = 1; q < 9; ++q) {
            const int xu = d2q9_xu(q), xv = d2q9_xv(q);
            const R wq = (R)d2q9_w(q);
            if (MODEL == AC) {
                dEqv[q] = wq * dp * P.invRT;
                fSov[q] = wq * ((sxf(xu, fx) + sxf(xv, fy)) * P.invRT);
                dhEqv[q] = wq * dphi_c;
            } else {
                const R u1 = (sxf(xu, U) + sxf(xv, V)) * P.invRT;
                const R G = u1 + R(0.5) * u1 * u1 - uu * P.Lambda0;
                const R cu = (R)xu - U, cv = (R)xv - V;
                dEqv[q] = wq * (dp + rho * G * P.RT);
                fSov[q] = wq * ((R(1.) + G) * (cu * fx + cv * fy) + G * P.RT * (cu * rhox + cv * rhoy));
                dhEqv[q] = wq * (dphi_c + u1 * phi);
            }
        }
        sEq = sym8(dEqv);
        shEq = sym8(dhEqv);
        dEqv[0] = (MODEL == AC ? R(0.) : dp) - sEq;
        dhEqv[0] = dphi_c - shEq;
        if (MODEL == AC) {
            fSov[0] = R(0.);
        } else {
            const R G0 = -uu * P.Lambda0;
            const R wq = (R)d2q9_w(0);
            fSov[0] = wq * ((R(1.) + G0) * (-U * fx - V * fy) + G0 * P.RT * (-U * rhox - V * rhoy));
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const int xu = d2q9_xu(q), xv = d2q9_xv(q);
            const R wq = (R)d2q9_w(q);
            const R hSo = (sxf(xu, srcx) + sxf(xv, srcy)) * wq;
            // collision increment B - T = (1-a)(Eq - T) + c S: small near equilibrium,
            // so B = T + increment keeps the rest state and rounds relative to the increment
            inc[q] = bBP * (dEqv[q] - df[q]) + cBP * fSov[q];
            inc[9 + q] = P.h_bBP * (dhEqv[q] - dh[q]) + P.h_cBP * hSo;
        }
        // the phase-field collision conserves sum_q h exactly (sum Eq = phi, sum S = 0):
        // the rest direction takes the exact negative of the others' increments
        inc[9] = -sym8(inc + 9);
        if (MODEL == HCZ) {
            // zeroth moment of the flow collision: (1-a)(p - sum f) + c sum S
            //   = (1-a) hDt RT (grad rho_old . u) + c RT (u . grad rho)
            inc[0] = (bBP * P.hDt * P.RT * (rxo_c * U + ryo_c * V) + cBP * P.RT * (U * rhox + V * rhoy)) -
                     sym8(inc);
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            sB[q][r][e] = df[q] + inc[q];
            sB[9 + q][r][e] = dh[q] + inc[9 + q];
        }
        sA[0][r][e] = srcx;
        sA[1][r][e] = srcy;
        sA[2][r][e] = rhox;
        sA[3][r][e] = rhoy;
        sA[4][r][e] = fx;
        sA[5][r][e] = fy;
    }
    if (WALLS) {
        __syncthreads();
        // P2: ghost rows of f-bar-plus and of the averaged fields (2 a0 - a1)
        if (act && ghost) {
            const int r0 = gj < 0 ? r + 1 : r - 1, r1 = gj < 0 ? r + 2 : r - 2;
#pragma unroll
            for (int k = 0; k < 18; ++k) sB[k][r][e] = R(2.) * sB[k][r0][e] - sB[k][r1][e];
#pragma unroll
            for (int k = 0; k < 6; ++k) sA[k][r][e] = R(2.) * sA[k][r0][e] - sA[k][r1][e];
        }
        // ghost phi for the next step's MacroSource, written by the tile owning the row
        if (real && e >= 1 && e <= w && r >= 1 && r <= hh) {
            if (gj == 0) S.gphi[(size_t)(gout * 2 + 0) * pitch + gi] = R(2.) * phi - sphi[r + 2][e + 1];
            if (gj == ny - 1) S.gphi[(size_t)(gout * 2 + 1) * pitch + gi] = R(2.) * phi - sphi[r][e + 1];
        }
    }
    __syncthreads();

    // ---- stage 2: west x-face and south y-face of this thread's cell
    R FW[18], FSo[18];
    const bool do_x = act && e >= 1 && r >= 1 && r <= hh;           // faces x0-1|x0 .. x0+w-1|x0+w
    const bool do_y = act && r >= 1 && e >= 1 && e <= w;            // faces below rows 0..hh (hh+1 with the top)
#pragma unroll
    for (int pass = 0; pass < 2; ++pass) {
        const bool xf = pass == 0;
        if (xf ? !do_x : !do_y) continue;
        // neighbours in the shared tile: x-face between (r, e-1) and (r, e);
        // y-face between (r-1, e) and (r, e)
        const int ro = xf ? r : r - 1, eo = xf ? e - 1 : e;
        R av[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) av[k] = R(0.5) * (sA[k][ro][eo] + sA[k][r][e]);
        R bh[18];
#pragma unroll
        for (int k = 0; k < 18; ++k) {
            const int q = k % 9;
            const R xu = (R)d2q9_xu(q), xv = (R)d2q9_xv(q);
            const R o = sB[k][ro][eo], n = sB[k][r][e];
            R gx, gy;
            if (xf) {
                gy = (R(0.5) * ((sB[k][r + 1][e] - sB[k][r - 1][e]) + (sB[k][r + 1][e - 1] - sB[k][r - 1][e - 1]))) * P.r_2dy;
                gx = (o - n) * P.r_ndx;
            } else {
                gx = (R(0.5) * ((sB[k][r][e - 1] - sB[k][r][e + 1]) + (sB[k][r - 1][e - 1] - sB[k][r - 1][e + 1]))) * P.r_n2dx;
                gy = (o - n) * P.r_ndy;
            }
            bh[k] = R(0.5) * (o + n) - P.hDt * (gx * xu + gy * xv);
        }
        // face moments
        // symmetric pairwise sums (0, E,NE,N,NW,W,SW,S,SE = 0..8)
        const R dphif = bh[9] + sym8(bh + 9);
        const R sf = (MODEL == AC ? R(0.) : bh[0]) + sym8(bh);
        const R su = (bh[1] - bh[5]) + ((bh[2] - bh[6]) + (bh[8] - bh[4]));
        const R sv = (bh[3] - bh[7]) + ((bh[2] - bh[6]) + (bh[4] - bh[8]));
        const R phif = P.phi0 + dphif;
        const R rhof = P.aPhi * phif + P.bPhi;
        R Uf, Vf, dpf, ah, bh_, ch;
        if (MODEL == AC) {
            Uf = R(0.);
            Vf = R(0.);
            dpf = sf * P.Kp;
            ah = P.ah_f;
        } else {
            const R inv = R(1.) / (rhof * P.RT);
            Uf = su * inv + R(0.5) * P.hDt * av[4] * inv;
            Vf = sv * inv + R(0.5) * P.hDt * av[5] * inv;
            dpf = sf + R(0.5) * P.hDt * P.RT * (av[2] * Uf + av[3] * Vf);
            ah = P.ah_f;
        }
        bh_ = R(1.) - ah;
        ch = P.tauf * bh_;
        const R uu = Uf * Uf + Vf * Vf;
        R out[18];
        R dEqv[9], fSov[9], dhEqv[9];
        R sEq, shEq;
#pragma unroll
        for (int q = 1; q < 9; ++q) {
            const int xu = d2q9_xu(q), xv = d2q9_xv(q);
            const R wq = (R)d2q9_w(q);
            if (MODEL == AC) {
                dEqv[q] = wq * dpf * P.invRT;
                fSov[q] = wq * ((sxf(xu, av[4]) + sxf(xv, av[5])) * P.invRT);
                dhEqv[q] = wq * dphif;
            } else {
                const R u1 = (sxf(xu, Uf) + sxf(xv, Vf)) * P.invRT;
                const R G = u1 + R(0.5) * u1 * u1 - uu * P.Lambda0;
                const R cu = (R)xu - Uf, cv = (R)xv - Vf;
                dEqv[q] = wq * (dpf + rhof * P.RT * G);
                fSov[q] = wq * ((R(1.) + G) * (cu * av[4] + cv * av[5]) + G * P.RT * (cu * av[2] + cv * av[3]));
                dhEqv[q] = wq * (dphif + u1 * phif);
            }
        }
        sEq = sym8(dEqv);
        shEq = sym8(dhEqv);
        dEqv[0] = (MODEL == AC ? R(0.) : dpf) - sEq;
        dhEqv[0] = dphif - shEq;
        if (MODEL == AC) {
            fSov[0] = R(0.);
        } else {
            const R G0 = -uu * P.Lambda0;
            const R wq = (R)d2q9_w(0);
            fSov[0] = wq * ((R(1.) + G0) * (-Uf * av[4] - Vf * av[5]) + G0 * P.RT * (-Uf * av[2] - Vf * av[3]));
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const int xu = d2q9_xu(q), xv = d2q9_xv(q);
            const R wq = (R)d2q9_w(q);
            const R hSo = (sxf(xu, av[0]) + sxf(xv, av[1])) * wq;
            out[9 + q] = dhEqv[q] + P.h_ah * (bh[9 + q] - dhEqv[q]) + P.h_ch * hSo;
            out[q] = dEqv[q] + ah * (bh[q] - dEqv[q]) + ch * fSov[q];
        }
        if (WALLS && !xf && (gj == 0 || gj == ny)) {
            // bounce-back of the directions entering the fluid (Ark/Cpp/Boundary.cpp:118-139)
            const bool bottom = gj == 0;
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                const int xv = d2q9_xv(q);
                if (bottom ? xv > 0 : xv < 0) {
                    out[q] = out[d2q9_bb(q)];
                    out[9 + q] = out[9 + d2q9_bb(q)];
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 18; ++k) {
            const int q = k % 9;
            const R v = sxf(xf ? d2q9_xu(q) : d2q9_xv(q), out[k]);
            if (xf) FW[k] = v;
            else FSo[k] = v;
        }
    }
    if (do_y) {
#pragma unroll
        for (int k = 0; k < 18; ++k) sFS[k][r][e] = FSo[k];
    }
    // east face = west face of the next lane
    R FE[18];
#pragma unroll
    for (int k = 0; k < 18; ++k) FE[k] = __shfl_down_sync(0xffffffffu, do_x ? FW[k] : R(0.), 1);
    __syncthreads();

    // ---- stage 3: finite-volume update of the interior cells (Update_phi_T) + aux
    if (real && e >= 1 && e <= w && r >= 1 && r <= hh) {
#pragma unroll
        for (int k = 0; k < 18; ++k) {
            // net flux with mirror-symmetric association
            const R s = (FW[k] - FE[k]) + (FSo[k] - sFS[k][r + 1][e]);
            const R dold = k < 9 ? df[k] : dh[k - 9];
            // 4/3 B - 1/3 T = T + (4/3)(B - T): old value plus one small increment,
            // rounded stochastically into storage
            const uint32_t key = (uint32_t)(c * 18 + k) * 0x9E3779B1U ^ (uint32_t)step * 0x85EBCA77U;
            const R dn = add_sr(dold, (inc[k] + P.bTP * inc[k]) + P.dtV * s, key);
            R *dst = k < 9 ? S.df : S.dh;
            dst[(size_t)(k % 9) * S.qs + c] = dn;
        }
        if (MODEL == AC) return;  // u = 0: the next step needs no previous force, gradient or phi*u
        S.aux[A_FX * S.qs + c] = fx;
        S.aux[A_FY * S.qs + c] = fy;
        S.aux[A_RHOX * S.qs + c] = rhox;
        S.aux[A_RHOY * S.qs + c] = rhoy;
        S.aux[A_PPU * S.qs + c] = phi * U;
        S.aux[A_PPV * S.qs + c] = phi * V;
    }
}

// Macroscopic fields of the FP32 state as FP64 arrays: the quantities the
// reference holds after Update_MacroVar + MacroSource of the last step.
template <int MODEL, bool WALLS, typename R>
__global__ void __launch_bounds__(256) k_macros32(PR<R> P, SR<R> S, double *rho_o, double *u_o, double *v_o,
                                                  double *p_o, double *phi_o, int opitch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= P.nx || j >= P.ny) return;
    const size_t c = (size_t)j * P.pitch + i;
    R df[9], dh[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        df[q] = S.df[(size_t)q * S.qs + c];
        dh[q] = S.dh[(size_t)q * S.qs + c];
    }
    R dphi, rho, U, V, dp;
    if (MODEL == AC)
        cell_macros<MODEL, R>(P, df, dh, R(0), R(0), R(0), R(0), dphi, rho, U, V, dp);
    else
        cell_macros<MODEL, R>(P, df, dh, S.aux[A_FX * S.qs + c], S.aux[A_FY * S.qs + c], S.aux[A_RHOX * S.qs + c],
                           S.aux[A_RHOY * S.qs + c], dphi, rho, U, V, dp);
    const size_t o = (size_t)j * opitch + i;
    rho_o[o] = (double)P.aPhi * ((double)P.phi0 + (double)dphi) + (double)P.bPhi;
    u_o[o] = U;
    v_o[o] = V;
    p_o[o] = (double)P.p0 + (double)dp;
    phi_o[o] = (double)P.phi0 + (double)dphi;
}

template <int MODEL, bool WALLS, typename R>
static cudaError_t launch_t(const PR<R> &P, const SR<R> &S, int first, int gin, int gout, cudaStream_t st,
                            uint32_t step) {
    const size_t bytes = SMEM_ELEMS * sizeof(R);
    static bool attr_set = false;  // per instantiation; idempotent, set before the first launch
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_step32<MODEL, WALLS, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)bytes);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const dim3 blk(BX, BY);
    const dim3 grd((P.nx + TW - 1) / TW, (P.ny + TH - 1) / TH);
    k_step32<MODEL, WALLS, R><<<grd, blk, bytes, st>>>(P, S, first, gin, gout, step);
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
