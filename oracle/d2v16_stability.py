"""Linear (von Neumann) stability of the DUGKS step with the D2V16 equilibrium --
TEST INFRASTRUCTURE ONLY (analysis for the tests and the design notes).

The reference's D2V16 model (Ark/Lib/D2V16.cpp, Ark/Lib/D2V16.h) has 16 velocities on
four rings (c, sqrt(2) c, 2c, 2 sqrt(2) c; the first ring carries the extra energy
variable eta = (3 + nK) c) and the equilibrium f_eq = M^-1 m(rho, u, v, T, p), m the 16
moments of Ark/Lib/D2V16.cpp:125-145 (Macro16).  Here M^-1 is the numerical inverse of
that moment basis (the closed-form table of Ark/Lib/D2V16.cpp:14-53 is its inverse;
tests/test_oracle_d2v16.py checks that), and the step is linearised around a uniform
state.

The step (Ark/Cpp/DUGKS2DSolver.cpp:175-295) on unit Cartesian cells, CD
reconstruction, no force:
  B   = a f + (1 - a) f_eq(f)                         a = (2 tau - h) / (2 tau + dt)
  f_f = a_h fb + (1 - a_h) f_eq(fb),  fb = L_q(B)      a_h = 2 tau / (2 tau + h)
  f'  = 4/3 B - 1/3 f + dt sum_faces (sign) xi.n f_f
with h = dt/2, dt = CFL / max|xi| (Ark/Constant/ZeroNamespace.h:12, D2V16.h MaxU =
2 sqrt(2) c), tau = nu / RT (Ark/Lib/D2Q9PP.cpp:39-42).  f_eq is linearised in (rho, j)
(isothermal closure: T = T0) or (rho, j, E) (thermal closure: T from the energy
moment, Ark/Lib/D2V16.cpp:187-198), by complex-step differentiation.  For a Fourier
mode exp(i k.x) the step is one 16x16 amplification matrix G(k); the scheme is stable
when the spectral radius of G stays <= 1 for every k.
"""
from __future__ import annotations

import numpy as np

RT0 = 1.0 / 3.0   # R0 T0 (Ark/Constant/ZeroReference.h:70-74)
DEGREES = 3.0     # 3 + nK, nK = 0 (Ark/Constant/ZeroReference.h:58)


def velocities(c: float):
    """(xi_u, xi_v, |xi|^2 + eta^2) of the D2V16 set with lattice speed c."""
    su = np.array([1, 0, -1, 0, 1, -1, -1, 1, 2, 0, -2, 0, 2, -2, -2, 2], float)
    sv = np.array([0, 1, 0, -1, 1, 1, -1, -1, 0, 2, 0, -2, 2, 2, -2, -2], float)
    e = DEGREES * c
    x2 = np.where(np.arange(16) < 4, c * c + e * e, (su * su + sv * sv) * c * c)
    return su * c, sv * c, x2


def basis(xu, xv, x2):
    """The 16 moment functions of Macro16's moments, evaluated at the 16 velocities."""
    return np.array([np.ones_like(xu), xu, xv, x2, xu * xv, xu ** 2, xv ** 2, xu * x2, xv * x2, xu ** 3, xv ** 3,
                     xu ** 2 * xv, xu * xv ** 2, xu * xv * x2, xu ** 2 * x2, xv ** 2 * x2])


def macro16(rho, u, v, RT):
    """Moments of the Maxwellian (Ark/Lib/D2V16.cpp:125-145) with p = rho RT."""
    D = DEGREES
    p = rho * RT
    u2, v2 = u * u, v * v
    s = u2 + v2
    return np.array([rho, rho * u, rho * v, rho * (D * RT + s), rho * u * v, rho * u2 + p, rho * v2 + p,
                     rho * u * ((D + 2) * RT + s), rho * v * ((D + 2) * RT + s), rho * u * (3 * RT + u2),
                     rho * v * (3 * RT + v2), rho * v * (RT + u2), rho * u * (RT + v2),
                     ((D + 4) * RT + s) * rho * u * v,
                     (D + 2) * rho * RT * RT + p * ((D + 5) * u2 + v2) + rho * u2 * s,
                     (D + 2) * rho * RT * RT + p * ((D + 5) * v2 + u2) + rho * v2 * s])


def rest_weights(c: float) -> np.ndarray:
    """f_eq(rho = 1, u = 0) at T0: one value per ring (rings of c, sqrt(2)c, 2c, 2 sqrt(2)c)."""
    xu, xv, x2 = velocities(c)
    f = np.linalg.solve(basis(xu, xv, x2), macro16(1.0, 0.0, 0.0, RT0))
    return f[[0, 4, 8, 12]]


def equilibrium_jacobian(c: float, u0: float = 0.0, v0: float = 0.0, thermal: bool = False) -> np.ndarray:
    """d f_eq / d f at the uniform state (rho = 1, u0, v0, T0), 16 x 16."""
    xu, xv, x2 = velocities(c)
    iM = np.linalg.inv(basis(xu, xv, x2))
    f0 = iM @ macro16(1.0, u0, v0, RT0)

    def feq(f):
        rho = f.sum()
        u = (f * xu).sum() / rho
        v = (f * xv).sum() / rho
        RT = RT0
        if thermal:
            RT = ((f * x2).sum() / rho - u * u - v * v) / DEGREES
        return iM @ macro16(rho, u, v, RT)

    W = np.empty((16, 16))
    hstep = 1e-30
    for k in range(16):
        d = np.zeros(16, complex)
        d[k] = 1j * hstep
        W[:, k] = np.imag(feq(f0.astype(complex) + d)) / hstep
    return W


def spectral_radius(c: float, nu: float, u0: float = 0.0, v0: float = 0.0, thermal: bool = False,
                    cfl: float = 0.5, nk: int = 24) -> float:
    """Largest |eigenvalue| of G(k) over an nk x nk grid of wave numbers (k = 0 excluded:
    there the conserved moments give eigenvalue 1 exactly)."""
    xu, xv, _ = velocities(c)
    W = equilibrium_jacobian(c, u0, v0, thermal)
    dt = cfl / (2.0 * np.sqrt(2.0) * c)
    h = 0.5 * dt
    tau = nu / RT0
    a = (2 * tau - h) / (2 * tau + dt)
    ah = 2 * tau / (2 * tau + h)
    I = np.eye(16)
    Ac = a * I + (1 - a) * W
    Af = ah * I + (1 - ah) * W
    ks = (np.arange(nk) + 0.5) * 2 * np.pi / nk - np.pi
    worst = 0.0
    for kx in ks:
        ex = np.exp(1j * kx)
        for ky in ks:
            ey = np.exp(1j * ky)
            # face values of a mode: average, normal gradient, tangential central differences
            phx = 0.5 * (1 + ex) - h * xu * (ex - 1) - h * xv * 0.5 * (1 + ex) * (1j * np.sin(ky))
            phy = 0.5 * (1 + ey) - h * xv * (ey - 1) - h * xu * 0.5 * (1 + ey) * (1j * np.sin(kx))
            G = (4.0 / 3.0) * Ac - I / 3.0 \
                + dt * (np.exp(-1j * kx) - 1) * np.diag(xu) @ Af @ np.diag(phx) @ Ac \
                + dt * (np.exp(-1j * ky) - 1) * np.diag(xv) @ Af @ np.diag(phy) @ Ac
            worst = max(worst, float(np.max(np.abs(np.linalg.eigvals(G)))))
    return worst


if __name__ == '__main__':
    for c in (0.5, 0.6, 0.7, 0.8, 1.0, 1.2):
        print(f'c = {c}: rest weights per ring {np.round(rest_weights(c), 4)}')
        for thermal in (False, True):
            row = ' '.join(f'nu={nu:g}:{spectral_radius(c, nu, thermal=thermal) - 1:+.1e}'
                           for nu in (0.01, 0.1, 0.3, 1.0, 10.0))
            print(f'   {"thermal" if thermal else "isothermal"}: max|lambda| - 1  {row}')
