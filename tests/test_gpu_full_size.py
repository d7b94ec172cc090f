"""The benchmark's own grid (8192 x 8192 Rayleigh-Taylor, HCZ, walls, FP32 storage) held to
size-independent properties, where no reference run of that size exists:
  * mirror symmetry: without the seeded noise the initial interface y = L (y_c + a cos(2 pi x
    / L)) is symmetric about x = L/2 (to the rounding of the FP64 cosine, ~1e-16), and every
    sum of the step is associated mirror-symmetrically, so after the steps rho, p, phi stay
    mirror images and u the negated mirror image to within FP32 rounding;
  * conservation: the phase field's and the density's domain sums stay within rounding of
    their initial values.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def rt8192():
    import bench
    from mpdugks_gb300 import capi
    wl = bench.WORKLOADS['rt8192']
    n = wl['nx']
    g = capi.GpuCase(capi.make_case('HCZ', 'fp32dev', **bench.case_kw(wl)), n, n, True)
    yc, amp = wl['init'][0], wl['init'][1]
    g.init('ac_rt', [yc, amp, 0.0])  # no noise: a mirror-symmetric interface
    r0 = g.reduce()
    g.step(30)
    yield g, r0
    g.close()


def test_full_size_mirror_symmetry(rt8192):
    g, _ = rt8192
    asym = {}
    for k in ('rho', 'p', 'phi', 'v'):
        a = g.get(k)
        asym[k] = float(np.max(np.abs(a - a[:, ::-1])) / np.max(np.abs(a)))
    u = g.get('u')
    umax = float(np.max(np.abs(u)))
    asym['u'] = float(np.max(np.abs(u + u[:, ::-1])) / umax)
    print('mirror asymmetry / max', asym, 'max|u|', umax)
    assert umax > 0.0  # the flow has started
    # measured after 30 steps: rho 6.3e-10, p 3.4e-12, phi 9.4e-10, u 2.7e-6, v 7.3e-7
    for k in ('rho', 'p', 'phi'):
        assert asym[k] <= 1e-8, (k, asym[k])
    for k in ('u', 'v'):
        assert asym[k] <= 3e-5, (k, asym[k])


def test_full_size_conservation(rt8192):
    g, r0 = rt8192
    r = g.reduce()
    assert abs(r.sum_phi - r0.sum_phi) <= 1e-12 * abs(r0.sum_phi)
    assert abs(r.sum_rho - r0.sum_rho) <= 1e-12 * abs(r0.sum_rho)
    assert g.check_finite() == 0
