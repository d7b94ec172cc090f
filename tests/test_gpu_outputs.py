"""Output quantities through the C ABI on the GPU: dugks_gpu_thermo_pressure and
dugks_gpu_drop_l2 against the numpy restatement (oracle/outputs.py) on the
handle's own fields.  Bit-exactness against the reference's printed values is
tested through dugks_run in test_host.py (the golden MidX / MidY / Diag files
and AC_Drop_L2Norm)."""
import numpy as np
import pytest

from oracle import outputs as O
from test_gpu_fp32 import make
from variants import VARIANTS

pytestmark = pytest.mark.gpu


def consts(v):
    c = v['consts']
    return O.constants(c['W'], c['Sigma'], c['RhoL'], c['RhoV'])


@pytest.mark.parametrize('name', ['hcz_drop', 'hcz_rt', 'ac_c1'])
@pytest.mark.parametrize('precision', ['fp64', 'fp32dev'])
def test_thermo_pressure_matches_the_oracle(name, precision):
    v = VARIANTS[name]
    gc = make(v, precision)
    gc.step(199)
    prev = gc.get('phi')
    gc.step(1)
    tp = gc.thermo_pressure()
    phi, p = gc.get('phi'), gc.get('p')
    if precision == 'fp64':
        # MacroSource's own gradient; wall ghosts extrapolated from the step's starting phi
        want = O.thermo_pressure(phi, p, consts(v), v['walls'], gc.get('rhox'), gc.get('rhoy'), ghost_phi=prev)
    else:  # the gradient from phi, with the same ghost rows
        want = O.thermo_pressure(phi, p, consts(v), v['walls'], ghost_phi=prev)
    assert np.max(np.abs(tp - want)) <= 1e-13 * np.max(np.abs(want)), name


@pytest.mark.parametrize('name', ['hcz_drop', 'ac_c1'])
@pytest.mark.parametrize('precision', ['fp64', 'fp32dev'])
def test_drop_l2_matches_the_oracle(name, precision):
    v = VARIANTS[name]
    gc = make(v, precision)
    l2_0 = gc.drop_l2()
    assert l2_0 <= 1e-15  # the initial field is the analytic profile
    gc.step(300)
    got = gc.drop_l2()
    want = O.drop_l2(gc.get('phi'), v['consts']['radius'], consts(v), inside=v['init'] == 'ac_drop_inside')
    assert got > 0 and abs(got - want) <= 1e-12 * want, (got, want)


def test_drop_l2_needs_a_drop():
    from mpdugks_gb300 import capi
    gc = make(VARIANTS['hcz_rt'], 'fp64')
    with pytest.raises(capi.DugksError):
        gc.drop_l2()
