"""FP32 deviation storage of the pseudopotential models (D2Q9PP, D2V16) against
the plain FP64 path.

Errors per field: max-norm and L2 ratios ||a - b|| / ||b|| over the grid.
Horizons: the D2Q9PP droplet is stable (2000 steps).  The D2V16 model (the
reference's D2V16 does not build; this is its restatement) diverges within a
few hundred steps in FP64 as well, at every tested setting (CPU restatement:
SCMP_Drop and seeded noise, T/Tc 0.7-0.85), so its comparison stops at 100
steps, before the divergence.  Phase separation from seeded noise amplifies
any perturbation (FP64 variants differ as well), so noise cases are compared
over 100 steps.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def pair(model, n, init, params):
    from mpdugks_gb300 import capi
    a = capi.GpuCase(capi.make_case(model, 'fp32dev'), n, n, False)
    b = capi.GpuCase(capi.make_case(model, 'fp64'), n, n, False)
    a.init(init, params, seed=7)
    b.init(init, params, seed=7)
    return a, b


def errors(a, b):
    out = {}
    for k in ('rho', 'u', 'v', 'p'):
        x, y = a.get(k), b.get(k)
        out[k] = (float(np.max(np.abs(x - y)) / np.max(np.abs(y))),
                  float(np.linalg.norm(x - y) / np.linalg.norm(y)))
    return out


@pytest.mark.parametrize('model,n,init,params,steps,tol', [
    # (rho max-norm, p max-norm, u/v L2)
    ('PP9', 32, 'scmp_drop', [], 2000, (1e-5, 5e-5, 5e-5)),
    ('PP9', 64, 'pp_noise', [0.2, 0.01], 100, (1e-5, 1e-5, 1e-4)),
    ('PP16', 32, 'scmp_drop', [], 100, (1e-5, 5e-5, 1e-4)),
    ('PP16', 64, 'pp_noise', [0.2, 0.01], 100, (1e-5, 1e-5, 1e-4)),
])
def test_fp32_pseudopotential_close_to_fp64(model, n, init, params, steps, tol):
    a, b = pair(model, n, init, params)
    a.step(steps)
    b.step(steps)
    e = errors(a, b)
    print(model, n, init, steps, {k: f'{v[0]:.2e}/{v[1]:.2e}' for k, v in e.items()})
    assert a.check_finite() == 0
    assert e['rho'][0] <= tol[0], e
    assert e['p'][0] <= tol[1], e
    assert e['u'][1] <= tol[2] and e['v'][1] <= tol[2], e


def test_fp32_pseudopotential_conserves_mass():
    from mpdugks_gb300 import capi
    g = capi.GpuCase(capi.make_case('PP9', 'fp32dev'), 48, 48, False)
    g.init('scmp_drop')
    m0 = g.reduce().sum_rho
    g.step(1000)
    m1 = g.reduce().sum_rho
    assert abs(m1 - m0) <= 1e-7 * m0


def test_fp32_pseudopotential_fields_and_distributions():
    """Distributions round-trip through the deviation storage; forces and psi are exposed."""
    from mpdugks_gb300 import capi
    a, b = pair('PP16', 32, 'scmp_drop', [])
    fa, fb = a.dist('f'), b.dist('f')
    assert np.max(np.abs(fa - fb)) <= 1e-7 * np.max(np.abs(fb))
    a.step(5)
    b.step(5)
    for k in ('fx', 'fy', 'psi'):
        x, y = a.get(k), b.get(k)
        assert np.max(np.abs(x - y)) <= 1e-4 * np.max(np.abs(y)), k


@pytest.mark.parametrize('precision', ['fp64', 'fp32dev'])
def test_d2v16_cases_of_different_lattice_speed_side_by_side(precision):
    """Each D2V16 case holds its own inverse moment matrix: two live cases with lattice
    speeds 0.5 and 0.6, stepped alternately, give what each gives alone."""
    from mpdugks_gb300 import capi

    def case(c):
        g = capi.GpuCase(capi.make_case('PP16', precision, d2v16_c=c), 32, 32, False)
        g.init('pp_noise', [0.2, 0.01], seed=5)
        return g
    alone = {}
    for c in (0.5, 0.6):
        g = case(c)
        g.step(20)
        alone[c] = {k: g.get(k) for k in ('rho', 'u', 'v')}
    a, b = case(0.5), case(0.6)
    for _ in range(10):
        a.step(2)
        b.step(2)
    for c, g in ((0.5, a), (0.6, b)):
        for k in ('rho', 'u', 'v'):
            assert np.array_equal(g.get(k), alone[c][k]), (c, k)
