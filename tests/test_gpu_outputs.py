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


def _laplace(model, precision, R, n=128, sigma=1e-2, mu=0.1, settle=20000, samples=10, every=250):
    """R dp / sigma of a resting drop, dp = mean p inside - mean p outside (cells more
    than 8 cells from the interface), averaged over `samples` snapshots; R from the
    drop's area (sum phi = pi R^2)."""
    from mpdugks_gb300 import capi
    gc = capi.GpuCase(capi.make_case(model, precision, Mu0=mu, M_Phi=0.1, W=4.0, Sigma=sigma, RhoL=10.0,
                                     RhoV=1.0), n, n, False)
    gc.init('ac_drop_inside', [float(R)])
    x = np.arange(n) + 0.5
    r = np.sqrt((x[None, :] - n / 2) ** 2 + (x[:, None] - n / 2) ** 2)
    gc.step(settle)
    ratios = []
    for _ in range(samples):
        gc.step(every)
        p, tp, phi = gc.get('p'), gc.thermo_pressure(), gc.get('phi')
        Reff = float(np.sqrt(np.sum(phi) / np.pi))
        ins, out = r < Reff - 8, r > Reff + 8
        # in the bulk phases thermoPressure reduces to p
        assert abs((tp[ins].mean() - tp[out].mean()) / (p[ins].mean() - p[out].mean()) - 1) < 0.02
        ratios.append((p[ins].mean() - p[out].mean()) * Reff / sigma)
    gc.close()
    return float(np.mean(ratios))


@pytest.mark.parametrize('precision', ['fp64', 'fp32dev'])
def test_laplace_law_hcz(precision):
    """Laplace's law dp = C sigma / R for resting HCZ drops of radius 16, 24 and 32
    (density ratio 10, Mu0 = 0.1): R dp is the same for every radius within 2 %.
    The coefficient C of the reference's HCZ pressure variable is not 1: it measures
    1.80 here (1.81 / 1.80 / 1.80, independent of the density ratio; the Allen-Cahn
    model with the same interface gives 0.93-0.95), so it is bounded, not pinned."""
    c = [_laplace('HCZ', precision, R) for R in (16, 24, 32)]
    print(precision, 'R dp / sigma', c)
    assert max(c) / min(c) - 1 < 0.02, c
    assert 1.5 < np.mean(c) < 2.1, c


def test_laplace_law_fp32_tracks_fp64():
    a, b = _laplace('HCZ', 'fp32dev', 24), _laplace('HCZ', 'fp64', 24)
    assert abs(a / b - 1) < 1e-4, (a, b)
