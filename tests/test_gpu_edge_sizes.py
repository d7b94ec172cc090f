"""Edge sizes: the smallest grids the ABI takes (3 cells across), odd and
non-square grids, grids narrower than a warp or a tile, with and without
walls.  The plain FP64 path must equal the oracle bit for bit; the FP32
storage path must stay within its tolerance of FP64."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

SIZES = [(3, 3), (5, 7), (8, 8), (33, 17), (65, 3), (3, 40)]
FIELDS = ('rho', 'u', 'v', 'p', 'phi')


def case_kw(model):
    return dict(Mu0=0.02, M_Phi=0.05, W=2.0, Sigma=1e-3, RhoL=3.0, RhoV=1.0,
                Gy=1e-4 if model == 'HCZ' else 0.0)


def init_of(nx, ny, walls):
    # a droplet of radius ~ a third of the grid, centred at (nx/2, nx/2) as the
    # reference's AC_Drop places it (walls: between the walls, under gravity)
    return 'ac_drop_inside', [max(1.0, min(nx, ny) / 3.0)]


@pytest.mark.parametrize('nx,ny', SIZES)
@pytest.mark.parametrize('model,walls', [('AC', False), ('HCZ', False), ('HCZ', True)])
def test_fp64_equals_the_oracle(nx, ny, model, walls):
    from mpdugks_gb300 import capi
    from oracle.oracle import Oracle
    if walls and ny < 3:
        pytest.skip('walls need three rows')
    kw = case_kw(model)
    init, params = init_of(nx, ny, walls)
    gc = capi.GpuCase(capi.make_case(model, 'fp64', **kw), nx, ny, walls)
    gc.init(init, params)
    o = Oracle(model, nx, ny, walls, init, radius=params[0], **kw)
    assert np.array_equal(gc.dist('f'), o.dists('f'))
    gc.step(30)
    o.step(30)
    for k in FIELDS:
        assert np.array_equal(gc.get(k), o.get(k)), (nx, ny, k)


UW_CODE = {'UW': 1, 'UW_LS': 2, 'UW_4P': 3}


@pytest.mark.parametrize('nx,ny', SIZES)
@pytest.mark.parametrize('scheme', ['UW', 'UW_LS', 'UW_4P'])
def test_fp64_uw_equals_the_oracle(nx, ny, scheme):
    """The upwind scheme with each cell gradient (periodic grids only) on the edge sizes:
    the plain FP64 path equals the oracle bit for bit."""
    from mpdugks_gb300 import capi
    from oracle.oracle import Oracle
    kw = case_kw('HCZ')
    init, params = init_of(nx, ny, False)
    gc = capi.GpuCase(capi.make_case('HCZ', 'fp64', scheme=scheme, **kw), nx, ny, False)
    gc.init(init, params)
    o = Oracle('HCZ', nx, ny, False, init, radius=params[0], uw=UW_CODE[scheme], **kw)
    gc.step(30)
    o.step(30)
    for k in FIELDS:
        assert np.array_equal(gc.get(k), o.get(k)), (nx, ny, k)


@pytest.mark.parametrize('nx,ny', SIZES)
def test_fp32_uw_close_to_fp64(nx, ny):
    """The FP32 upwind step (four launches, any grid size) against FP64 UW from a seeded
    noisy interface, as the central-scheme test below."""
    from mpdugks_gb300 import capi
    kw = case_kw('HCZ')
    out = {}
    for prec in ('fp32dev', 'fp64'):
        g = capi.GpuCase(capi.make_case('HCZ', prec, scheme='UW', **kw), nx, ny, False)
        g.init('ac_rt', [0.5 * ny / nx, 0.1, 1e-3], seed=5)
        g.step(30)
        assert g.check_finite() == 0
        out[prec] = {k: g.get(k) for k in FIELDS}
    for k in ('rho', 'p', 'phi'):
        assert rel_err(out['fp32dev'][k], out['fp64'][k]) <= 2e-5, (nx, ny, k)


@pytest.mark.parametrize('nx,ny', SIZES)
@pytest.mark.parametrize('model,walls', [('AC', False), ('HCZ', True)])
def test_fused_kernel_equals_fp64_to_rounding(nx, ny, model, walls):
    """The fused deviation-form kernels (tile and halo wrap logic) carried out in
    FP64 against the plain FP64 path on the same symmetric droplets."""
    from mpdugks_gb300 import capi
    kw = case_kw(model)
    init, params = init_of(nx, ny, walls)
    out = {}
    for prec in ('fp64fused', 'fp64'):
        g = capi.GpuCase(capi.make_case(model, prec, **kw), nx, ny, walls)
        g.init(init, params)
        g.step(30)
        out[prec] = {k: g.get(k) for k in FIELDS}
    for k in ('rho', 'p', 'phi'):
        assert rel_err(out['fp64fused'][k], out['fp64'][k]) <= 1e-13, (nx, ny, k)


@pytest.mark.parametrize('nx,ny', SIZES)
@pytest.mark.parametrize('model,walls', [('AC', False), ('HCZ', True)])
def test_fp32_close_to_fp64(nx, ny, model, walls):
    """FP32 storage against FP64 from a seeded noisy interface.  (A symmetric
    droplet on a 3x3 or 5x7 grid has cells where the FP64 phase gradient is
    exactly zero and the FP32 one a rounding-level nonzero: the reference's
    MacroSource clamps the one and normalises the other, an O(1) difference of
    the source at that cell -- the discontinuity of its algorithm, not of the
    storage.)"""
    from mpdugks_gb300 import capi
    kw = case_kw(model)
    init, params = 'ac_rt', [0.5 * ny / nx, 0.1, 1e-3]
    out = {}
    for prec in ('fp32dev', 'fp64'):
        g = capi.GpuCase(capi.make_case(model, prec, **kw), nx, ny, walls)
        g.init(init, params, seed=5)
        g.step(30)
        assert g.check_finite() == 0
        out[prec] = {k: g.get(k) for k in FIELDS}
    for k in ('rho', 'p', 'phi'):
        assert rel_err(out['fp32dev'][k], out['fp64'][k]) <= 2e-5, (nx, ny, k)
