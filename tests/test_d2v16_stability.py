"""The D2V16 lattice at the reference's speed c = 1.2 (Ark/Lib/D2V16.h MaSpan, with
T0 = 1/3) is linearly unstable in the DUGKS step for relaxation times tau = nu/RT above
~0.3, with either closure of the temperature; at c = 0.5 the step is stable over the
relaxation times a liquid-vapour case spans (nu = Mu0 / rho up to ~10 in the vapour),
at rest and in a uniform flow.  The analysis is oracle/d2v16_stability.py (von Neumann,
linearised around a uniform state); these checks pin it and the velocity set it uses."""
import numpy as np
import pytest

from oracle import d2v16_stability as st
from oracle.oracle import Oracle


@pytest.mark.parametrize('c', [0.5, 1.2])
def test_velocity_set_is_the_oracles(c):
    o = Oracle('PP16', 8, 8, init='pp_noise', d2v16_c=c)
    for a, b in zip(st.velocities(c), o.velocities()):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-15)
    # the numerical inverse of the moment basis is the restated closed-form equilibrium
    xu, xv, x2 = st.velocities(c)
    f = np.linalg.solve(st.basis(xu, xv, x2), st.macro16(0.3, 0.05, -0.02, st.RT0))
    np.testing.assert_allclose(f, o.d2v16_equilibrium(0.3, 0.05, -0.02), rtol=1e-11, atol=1e-14)


def test_rest_equilibrium_has_a_negative_ring():
    w = st.rest_weights(1.2)
    assert abs(w.sum() * 4 - 1.0) < 1e-12
    assert w[2] < -0.35  # the 2c axis ring
    assert st.rest_weights(0.5)[2] < 0  # negative at c = 0.5 too: positivity is not what decides


@pytest.mark.parametrize('thermal,nu', [(False, 0.1), (False, 1.0), (True, 0.3)])
def test_reference_lattice_speed_is_unstable(thermal, nu):
    # growth of at least 0.5 % per step for some wave number (1 % on the finer grid)
    assert st.spectral_radius(1.2, nu, thermal=thermal, nk=24) > 1.005


@pytest.mark.parametrize('nu', [0.01, 0.1, 1.0, 10.0])
@pytest.mark.parametrize('u0,v0', [(0.0, 0.0), (0.1, 0.05)])
def test_half_lattice_speed_is_stable(nu, u0, v0):
    assert st.spectral_radius(0.5, nu, u0, v0, nk=16) <= 1.0 + 1e-12
