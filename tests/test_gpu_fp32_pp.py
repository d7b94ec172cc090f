"""FP32 storage of the pseudopotential models (D2Q9PP, D2V16) against the plain FP64
path.

Errors per field: max-norm and L2 ratios ||a - b|| / ||b|| over the grid.  The
resting droplets are held to 1e-5 in the max-norm on every field over 2000 steps.
D2V16 runs at the lattice speed c = 0.5: at the reference's c = 1.2 (T0 = 1/3) the
rest equilibrium of the 2c axis ring is -0.36 rho and the linearised step is unstable
for relaxation times above ~0.3 (tests/test_d2v16_stability.py), so a droplet there
diverges within a few hundred steps in FP64 as well.  Phase separation from seeded
noise amplifies any perturbation, rounding included: those cases are compared
against the spread that two FP64 evaluations (plain and FMA-contracted) already show.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def pair(model, n, init, params, precisions=('fp32dev', 'fp64'), **kw):
    from mpdugks_gb300 import capi
    out = []
    for prec in precisions:
        g = capi.GpuCase(capi.make_case(model, prec, **kw), n, n, False)
        g.init(init, params, seed=7)
        out.append(g)
    return out


def errors(a, b):
    out = {}
    for k in ('rho', 'u', 'v', 'p'):
        x, y = a.get(k), b.get(k)
        out[k] = (float(np.max(np.abs(x - y)) / np.max(np.abs(y))),
                  float(np.linalg.norm(x - y) / np.linalg.norm(y)))
    return out


@pytest.mark.parametrize('model,kw', [('PP9', {}), ('PP16', dict(d2v16_c=0.5))])
def test_fp32_pseudopotential_droplet_within_target(model, kw):
    a, b = pair(model, 32, 'scmp_drop', [], **kw)
    a.step(2000)
    b.step(2000)
    e = errors(a, b)
    print(model, {k: f'{v[0]:.2e}/{v[1]:.2e}' for k, v in e.items()})
    assert a.check_finite() == 0
    for k in ('rho', 'p', 'u', 'v'):
        assert e[k][0] <= 1e-5, (k, e)


@pytest.mark.parametrize('model,kw', [('PP9', {}), ('PP16', dict(d2v16_c=0.5))])
def test_fp32_pseudopotential_noise_within_fp64_spread(model, kw):
    """Spinodal growth from 1 % density noise (100 steps): FP32 storage against FP64 is
    within the target on rho and p, and its velocity difference is of the size that the
    FMA-contracted FP64 variant already shows against plain FP64."""
    a, b, c = pair(model, 64, 'pp_noise', [0.2, 0.01], ('fp32dev', 'fp64', 'fp64fma'), **kw)
    for g in (a, b, c):
        g.step(100)
    e, efma = errors(a, b), errors(c, b)
    print(model, {k: f'{v[0]:.2e}/{v[1]:.2e}' for k, v in e.items()},
          'fma', {k: f'{v[0]:.2e}/{v[1]:.2e}' for k, v in efma.items()})
    assert a.check_finite() == 0
    assert e['rho'][0] <= 1e-5 and e['p'][0] <= 1e-5, e
    for k in ('u', 'v'):
        assert e[k][0] <= max(1e-5, 10 * efma[k][0]), (k, e, efma)


def test_fp32_pseudopotential_conserves_mass():
    from mpdugks_gb300 import capi
    g = capi.GpuCase(capi.make_case('PP9', 'fp32dev'), 48, 48, False)
    g.init('scmp_drop')
    m0 = g.reduce().sum_rho
    g.step(1000)
    m1 = g.reduce().sum_rho
    assert abs(m1 - m0) <= 1e-7 * m0


def test_fp32_pseudopotential_fields_and_distributions():
    """Distributions round-trip through the storage (rho in FP64 plus FP32 remainders);
    forces and psi are exposed."""
    a, b = pair('PP16', 32, 'scmp_drop', [], d2v16_c=0.5)
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


def _handle(model, nx, ny, init, params, passes=None, **kw):
    """A FP32 pseudopotential handle; passes=1 selects the single-pass step form."""
    import os
    from mpdugks_gb300 import capi
    old = os.environ.pop('DUGKS_PP_PASSES', None)
    if passes:
        os.environ['DUGKS_PP_PASSES'] = str(passes)
    try:
        g = capi.GpuCase(capi.make_case(model, 'fp32dev', **kw), nx, ny, False)
    finally:
        os.environ.pop('DUGKS_PP_PASSES', None)
        if old is not None:
            os.environ['DUGKS_PP_PASSES'] = old
    g.init(init, params, seed=11)
    return g


@pytest.mark.parametrize('model,kw', [('PP9', {}), ('PP16', dict(d2v16_c=0.5))])
@pytest.mark.parametrize('nx,ny,init,params', [(64, 40, 'pp_noise', [0.2, 0.01]), (33, 8, 'pp_noise', [0.2, 0.01]),
                                               (96, 160, 'scmp_drop', []), (300, 270, 'pp_noise', [0.13044, 0.01])])
def test_single_pass_step_equals_three_passes(model, kw, nx, ny, init, params):
    """The single-pass streaming step against the three-pass step on grids of one or
    several strips and segments (26-column strips, ragged last strip, 8 rows = the
    smallest grid it takes): the same arithmetic, so the same fields and remainders."""
    if model == 'PP16' and init == 'pp_noise':
        params = [0.13044, 0.01]
    a = _handle(model, nx, ny, init, params, passes=1, **kw)
    b = _handle(model, nx, ny, init, params, **kw)
    for steps in (1, 7):
        a.step(steps)
        b.step(steps)
        for k in ('rho', 'u', 'v', 'p', 'psi', 'fx', 'fy'):
            x, y = a.get(k), b.get(k)
            assert np.array_equal(x, y), (k, float(np.max(np.abs(x - y))))
        assert np.array_equal(a.dist('f'), b.dist('f'))
