"""Output quantities of the Allen-Cahn models in numpy -- TEST INFRASTRUCTURE ONLY
(the checker of dugks_gpu_drop_l2 / dugks_gpu_thermo_pressure; the product never
imports it).

  drop_l2          AC_Drop_L2Norm (Ark/Cpp/Output.cpp:226-238) with the profile of
                   AnalyticalPhiAC_Drop (Ark/Cpp/Preprocess.cpp:402-438)
  thermo_pressure  thermoPressure (Ark/Cpp/Output.cpp:146-163) with the gradient of
                   update_MQ_x / update_MQ_y (Ark/Lib/GradSchemeBasic.h:153-180,
                   apsi = 4, bpsi = 1, SetZero below 1e-14), Rho_x = aPhi Phi_x
                   (MacroSource), and the 9-point Laplacian of update_Laplacian_Phi
                   (Ark/Cpp/GradScheme.cpp:347-365)
  constants        the phase-field constants of Ark/Constant/ZeroNamespace.h
                   (Beta = 12 sigma / W, Kappa = 3 sigma W / 2, PhiL = 1, PhiV = 0,
                   aPhi = RhoL - RhoV)

Cells are [ny][nx] arrays, cell (i, j) centred at (i + 1/2, j + 1/2); grids are
periodic in x, and in y unless ``walls`` gives the ghost rows below row 0 and
above row ny - 1: 2 phi_0 - phi_1 and 2 phi_{ny-1} - phi_{ny-2} of ``ghost_phi``.
The reference extrapolates its wall shadow cells in the collision stage
(Ark/Cpp/Boundary.cpp:38-63, called at Ark/Cpp/DUGKS2DSolver.cpp:188), from the
phase field the step started with, and the MacroSource at the step's end reads
them: ``ghost_phi`` is that field (the previous step's), ``phi`` by default.
"""
from __future__ import annotations

import numpy as np


def constants(W: float, Sigma: float, RhoL: float, RhoV: float) -> dict:
    return dict(Beta=12 * Sigma / W, Kappa=3 * Sigma * W / 2, PhiL=1.0, PhiV=0.0, aPhi=RhoL - RhoV, wI=W,
                MinL=1.0, dx2=2.0)


def drop_profile(nx: int, ny: int, radius: float, k: dict, inside: bool = False) -> np.ndarray:
    x = np.arange(nx) + 0.5
    y = np.arange(ny)[:, None] + 0.5
    c = 0.5 * nx
    r = np.sqrt((x - c) * (x - c) + (y - c) * (y - c))
    d = (radius - r) if inside else (r - radius)
    return 0.5 * (k['PhiL'] + k['PhiV']) + 0.5 * (k['PhiL'] - k['PhiV']) * np.tanh(d * 2 / k['wI'])


def drop_l2(phi: np.ndarray, radius: float, k: dict, inside: bool = False) -> float:
    a = drop_profile(phi.shape[1], phi.shape[0], radius, k, inside)
    d = phi - a
    # the reference's sums run cell by cell; a sequential sum in float64
    sd, sa = 0.0, 0.0
    for dv, av in zip(d.ravel().tolist(), a.ravel().tolist()):
        sd += dv * dv
        sa += av * av
    return float(np.sqrt(sd / sa))


def _padded(phi: np.ndarray, walls: bool, ghost_phi: np.ndarray | None = None) -> np.ndarray:
    ny, nx = phi.shape
    P = np.empty((ny + 2, nx + 2))
    P[1:-1, 1:-1] = phi
    if walls:
        g = phi if ghost_phi is None else ghost_phi
        P[0, 1:-1] = 2.0 * g[0] - g[1]
        P[-1, 1:-1] = 2.0 * g[-1] - g[-2]
    else:
        P[0, 1:-1] = phi[-1]
        P[-1, 1:-1] = phi[0]
    P[:, 0] = P[:, -2]
    P[:, -1] = P[:, 1]
    return P


def phase_gradient(phi: np.ndarray, k: dict, walls: bool = False,
                   ghost_phi: np.ndarray | None = None) -> tuple[np.ndarray, np.ndarray]:
    """Rho_x, Rho_y of MacroSource: aPhi times the SetZero'd isotropic gradient of phi."""
    P = _padded(phi, walls, ghost_phi)
    E, W, N, S = P[1:-1, 2:], P[1:-1, :-2], P[2:, 1:-1], P[:-2, 1:-1]
    NE, NW, SW, SE = P[2:, 2:], P[2:, :-2], P[:-2, :-2], P[:-2, 2:]
    gx = (4 * (E - W) + 1 * (NE - NW + SE - SW)) / (k['dx2'] * 6)
    gy = (4 * (N - S) + 1 * (NE - SE + NW - SW)) / (k['dx2'] * 6)
    gx = np.where(np.abs(gx) < 1e-14, 0.0, gx)
    gy = np.where(np.abs(gy) < 1e-14, 0.0, gy)
    return k['aPhi'] * gx, k['aPhi'] * gy


def laplacian(phi: np.ndarray, k: dict, walls: bool = False, ghost_phi: np.ndarray | None = None) -> np.ndarray:
    P = _padded(phi, walls, ghost_phi)
    E, W, N, S = P[1:-1, 2:], P[1:-1, :-2], P[2:, 1:-1], P[:-2, 1:-1]
    NE, NW, SW, SE = P[2:, 2:], P[2:, :-2], P[:-2, :-2], P[:-2, 2:]
    return (4 * (E + N + W + S) + (NE + NW + SW + SE) - 20 * phi) / (6 * k['MinL'] * k['MinL'])


def thermo_pressure(phi: np.ndarray, p: np.ndarray, k: dict, walls: bool = False,
                    rho_x: np.ndarray | None = None, rho_y: np.ndarray | None = None,
                    ghost_phi: np.ndarray | None = None) -> np.ndarray:
    if rho_x is None or rho_y is None:
        rho_x, rho_y = phase_gradient(phi, k, walls, ghost_phi)
    B, K, L, V, a = k['Beta'], k['Kappa'], k['PhiL'], k['PhiV'], k['aPhi']
    sq = (rho_x * rho_x + rho_y * rho_y) / (a * a)
    p0 = phi * 2 * B * (phi - L) * (phi - V) * (2 * phi - L - V) - B * (phi - L) * (phi - L) * (phi - V) * (phi - V)
    return p0 - K * phi * laplacian(phi, k, walls, ghost_phi) + K * sq / 2 + p
