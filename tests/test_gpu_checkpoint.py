"""Checkpoint / restart (dugks_gpu_checkpoint / dugks_gpu_restore): a run of N
steps and a run of N/2 steps, checkpoint, a new handle restored from it and
N/2 more steps give bit-identical states, for every precision and model."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ('rho', 'u', 'v', 'p', 'phi')

CASES = [
    ('AC', 'fp64', 40, 32, False, 'ac_drop_inside', [10.0], {}),
    ('HCZ', 'fp64', 16, 64, True, 'ac_rt', [1.0, 0.1, 1e-4], dict(Gy=1e-4, RhoL=3.0, RhoV=1.0)),
    ('HCZ', 'fp64fma', 32, 32, False, 'ac_drop_inside', [8.0], dict(scheme='UW')),
    ('HCZ', 'fp64', 24, 48, True, 'ac_rt', [1.0, 0.1, 1e-4], dict(Gy=1e-4, RhoL=3.0, RhoV=1.0, wall='NEE')),
    ('HCZ', 'fp32dev', 64, 96, True, 'ac_rt', [1.0, 0.1, 1e-4], dict(Gy=1e-4, RhoL=3.0, RhoV=1.0)),
    # enough strip segments for the streaming kernel (the small FP32 grids run the tile kernel)
    ('HCZ', 'fp32dev', 1120, 1664, True, 'ac_rt', [1.0, 0.1, 1e-4], dict(Gy=1e-4, RhoL=3.0, RhoV=1.0)),
    ('HCZ', 'fp64fused', 48, 48, False, 'ac_drop_inside', [12.0], {}),
    ('PP16', 'fp32dev', 32, 32, False, 'scmp_drop', [], {}),
    # the upwind scheme in FP32 storage (its scratch is rebuilt every step) and the
    # least-squares cell gradient in FP64
    ('HCZ', 'fp32dev', 40, 36, False, 'ac_drop_inside', [9.0], dict(scheme='UW')),
    ('AC', 'fp64', 24, 20, False, 'ac_drop_inside', [6.0], dict(scheme='UW_LS')),
    ('PP9', 'fp64', 32, 32, False, 'scmp_drop', [], {}),
]


def make(model, prec, nx, ny, walls, kw):
    from mpdugks_gb300 import capi
    base = dict(Mu0=0.01, M_Phi=0.05, W=4.0, Sigma=1e-3, RhoL=1.0, RhoV=0.1) if model in ('AC', 'HCZ') else {}
    base.update(kw)
    return capi.GpuCase(capi.make_case(model, prec, **base), nx, ny, walls)


@pytest.mark.parametrize('model,prec,nx,ny,walls,init,params,kw', CASES)
@pytest.mark.parametrize('first_half', [7, 10])
def test_restart_is_bit_identical(model, prec, nx, ny, walls, init, params, kw, first_half):
    n = 20
    a = make(model, prec, nx, ny, walls, kw)
    a.init(init, params, seed=3)
    a.step(n)
    b = make(model, prec, nx, ny, walls, kw)
    b.init(init, params, seed=3)
    b.step(first_half)
    ck = b.checkpoint()
    b.close()
    c = make(model, prec, nx, ny, walls, kw)
    c.restore(ck)
    c.step(n - first_half)
    for k in FIELDS:
        assert np.array_equal(a.get(k), c.get(k)), k
    assert np.array_equal(a.dist('f'), c.dist('f'))
    assert a.reduce().steps == c.reduce().steps == n


def test_restore_refuses_another_case():
    from mpdugks_gb300 import capi
    a = make('AC', 'fp64', 40, 32, False, {})
    a.init('ac_drop_inside', [10.0])
    ck = a.checkpoint()
    other = make('AC', 'fp64', 40, 33, False, {})
    with pytest.raises(capi.DugksError) as e:
        other.restore(ck)
    assert e.value.code == capi.DUGKS_EINVAL and 'different case' in str(e.value)
    bad = ck.copy()
    bad[:8] = 0
    with pytest.raises(capi.DugksError):
        a.restore(bad)
    with pytest.raises(capi.DugksError):
        a.restore(ck[:100])


def test_driver_resumes_from_a_checkpoint(tmp_path):
    """dugks_run on the reference's AC_Drop 32x24 Case.ark: 20 steps in one run, or 10
    steps with a checkpoint and a resumed run to 20: the step-20 FlowField files are
    byte-identical, and equal to the reference's own."""
    import gzip
    import subprocess
    from pathlib import Path
    from mpdugks_gb300 import build
    build.build()
    gold = Path(__file__).resolve().parent / 'golden' / 'flowfield' / 'ac_ff'
    run = [str(build.RUNNER), 'run', str(gold / 'Case.ark')]
    subprocess.run(run + ['--out', str(tmp_path / 'a'), '--steps', '20'], check=True, capture_output=True)
    ck = tmp_path / 'state.ck'
    subprocess.run(run + ['--out', str(tmp_path / 'b'), '--steps', '10', '--checkpoint', str(ck)], check=True,
                   capture_output=True)
    r = subprocess.run(run + ['--out', str(tmp_path / 'c'), '--steps', '20', '--resume', str(ck)], check=True,
                       capture_output=True, text=True)
    assert 'resumed' in r.stdout and 'step 10' in r.stdout
    f = next(gold.glob('step20Ma*.dat.gz'))
    name = f.name[:-3]
    a = (tmp_path / 'a' / 'global' / name).read_bytes()
    c = (tmp_path / 'c' / 'global' / name).read_bytes()
    assert a == c == gzip.decompress(f.read_bytes())
