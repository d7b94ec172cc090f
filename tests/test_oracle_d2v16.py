"""Known-answer tests of the restated D2V16 model (the reference's
Ark/Lib/D2V16.cpp does not compile, so no reference binary pins it).

Its equilibrium is the inverse moment matrix (Ark/Lib/D2V16.cpp:14-53) applied
to the 16 moments of Macro16 (:125-145), the moments of a Maxwellian with
D = 3 degrees of freedom (two translational, one internal through eta) at
p = rho R T.  The moment basis psi_k(xi) follows from those moments:
1, xi_x, xi_y, |xi|^2 + eta^2, xi_x xi_y, xi_x^2, xi_y^2, xi_x (|xi|^2 + eta^2),
xi_y (|xi|^2 + eta^2), xi_x^3, xi_y^3, xi_x^2 xi_y, xi_x xi_y^2,
xi_x xi_y (|xi|^2 + eta^2), xi_x^2 (|xi|^2 + eta^2), xi_y^2 (|xi|^2 + eta^2).
The GPU FP64 D2V16 path equals this oracle bit for bit
(tests/test_gpu_parity.py::test_d2v16_pseudopotential_matches_oracle), so these
checks cover it too."""
import numpy as np
import pytest

from oracle.oracle import Oracle


def basis(xu, xv, x2):
    return np.array([np.ones_like(xu), xu, xv, x2, xu * xv, xu ** 2, xv ** 2, xu * x2, xv * x2, xu ** 3, xv ** 3,
                     xu ** 2 * xv, xu * xv ** 2, xu * xv * x2, xu ** 2 * x2, xv ** 2 * x2])


def maxwell_moments(rho, u, v, RT, D=3.0):
    p = rho * RT
    u2, v2, s2 = u * u, v * v, u * u + v * v
    return np.array([
        rho, rho * u, rho * v, rho * (D * RT + s2), rho * u * v, rho * u2 + p, rho * v2 + p,
        rho * u * ((D + 2) * RT + s2), rho * v * ((D + 2) * RT + s2),
        rho * u * (3 * RT + u2), rho * v * (3 * RT + v2), rho * v * (RT + u2), rho * u * (RT + v2),
        ((D + 4) * RT + s2) * rho * u * v,
        (D + 2) * rho * RT * RT + p * ((D + 5) * u2 + v2) + rho * u2 * s2,
        (D + 2) * rho * RT * RT + p * ((D + 5) * v2 + u2) + rho * v2 * s2,
    ])


@pytest.mark.parametrize('c', [1.2, 1.0])
def test_equilibrium_has_the_maxwellian_moments(c):
    o = Oracle('PP16', 8, 8, init='pp_noise', d2v16_c=c)
    xu, xv, x2 = o.velocities()
    RT = o.const('RT')
    Psi = basis(xu, xv, x2)
    rng = np.random.default_rng(7)
    for _ in range(20):
        rho, u, v = rng.uniform(0.05, 1.0), rng.uniform(-0.1, 0.1), rng.uniform(-0.1, 0.1)
        feq = o.d2v16_equilibrium(rho, u, v)
        got = Psi @ feq
        want = maxwell_moments(rho, u, v, RT)
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-13 * rho)


def test_inverse_matrix_inverts_the_basis():
    """The closed-form coefficients restated from the reference give the inverse of
    the moment basis: feq(rho, u, v) is linear in the 16 moments with the matrix
    Psi^-1, checked column by column through the equilibria of 16 moment vectors."""
    o = Oracle('PP16', 8, 8, init='pp_noise')
    xu, xv, x2 = o.velocities()
    Psi = basis(xu, xv, x2)
    assert np.linalg.cond(Psi) < 1e6
    RT = o.const('RT')
    rng = np.random.default_rng(3)
    for _ in range(5):
        rho, u, v = rng.uniform(0.1, 1.0), rng.uniform(-0.2, 0.2), rng.uniform(-0.2, 0.2)
        feq = o.d2v16_equilibrium(rho, u, v)
        np.testing.assert_allclose(feq, np.linalg.solve(Psi, maxwell_moments(rho, u, v, RT)), rtol=1e-10,
                                   atol=1e-13)


def test_periodic_run_conserves_mass():
    o = Oracle('PP16', 24, 20, init='pp_noise', noise_rho0=0.2, noise_amp=0.01, seed=9)
    m0 = o.get('rho').sum()
    o.step(60)
    m1 = o.get('rho').sum()
    assert abs(m1 - m0) <= 1e-12 * m0


def opposite(q):
    return (q & ~3) | ((q + 2) & 3)


def entry(j, k):
    """Entries of the inverse moment matrix that are not identically zero (the axis rings'
    rows, directions 0-3 and 8-11, have none at the moments 1, 2, 4, 13 and, along x,
    8, 10, 11; along y, 7, 9, 12): the structure the GPU equilibria skip."""
    if j & 4:
        return True
    return k not in ((1, 2, 4, 13) + ((7, 9, 12) if j & 1 else (8, 10, 11)))


ODD = (1, 2, 7, 8, 9, 10, 11, 12)


@pytest.mark.parametrize('c', [1.2, 0.5])
def test_inverse_moment_matrix_has_the_pair_form(c):
    """Row q' (the opposite direction) of the inverse moment matrix equals row q in the
    moments even in xi and is its negation in the odd ones; the zeros sit where entry()
    says.  The FP32 and FP64-FMA equilibria evaluate the matrix by these pairs, and every
    handle checks its own table for this form when it is made."""
    o = Oracle('PP16', 8, 8, init='pp_noise', d2v16_c=c)
    xu, xv, x2 = o.velocities()
    for q in range(16):
        assert xu[opposite(q)] == -xu[q] and xv[opposite(q)] == -xv[q]
    iM = np.linalg.inv(basis(xu, xv, x2))  # iM[q, k]
    scale = np.abs(iM).max(axis=0)
    for j in range(16):
        jo = opposite(j)
        for k in range(16):
            if not entry(j, k):
                assert abs(iM[j, k]) <= 1e-12 * scale[k], (j, k)
            sign = -1.0 if k in ODD else 1.0
            assert abs(iM[jo, k] - sign * iM[j, k]) <= 1e-12 * scale[k], (j, k)


def test_equilibrium_reverses_with_the_velocity():
    """eq_q(rho, -u, -v) == eq_q'(rho, u, v) bit for bit: the moments change sign exactly
    with (u, v) and the oracle's table has the pair form."""
    o = Oracle('PP16', 8, 8, init='pp_noise', d2v16_c=0.5)
    rng = np.random.default_rng(11)
    opp = [opposite(q) for q in range(16)]
    for _ in range(50):
        rho, u, v = rng.uniform(0.01, 0.4), rng.uniform(-0.2, 0.2), rng.uniform(-0.2, 0.2)
        a = o.d2v16_equilibrium(rho, u, v)
        b = o.d2v16_equilibrium(rho, -u, -v)
        assert np.array_equal(b, a[opp])
