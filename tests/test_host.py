"""Host side of the drop-in: Case.ark reader/writer, FlowField and line-profile
writers and the dugks_run driver, against files written by the reference's own
OutputCase, Output_Flowfield, Output_MidX / MidY / Diag and AC_Drop_L2Norm
(tests/golden/flowfield, made by make_flowfield_golden.py)."""
import gzip
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLD = ROOT / 'tests' / 'golden' / 'flowfield'
CASES = ['ac_ff', 'hcz_rt', 'uw_ff', 'nee_rt']


def runner() -> Path:
    from mpdugks_gb300 import build
    build.build()
    return build.RUNNER


def golden_dat(case: str, step: int) -> tuple[str, bytes]:
    f = next(GOLD.joinpath(case).glob(f'step{step}Ma*.dat.gz'))
    return f.name[:-3], gzip.decompress(f.read_bytes())


def parse_flowfield(text: bytes, cells: int) -> dict[str, np.ndarray]:
    lines = text.decode().splitlines()
    out, k = {}, 0
    for name in ('rho', 'uv', 'p', 'T', 'phi', 'tau', 'fx', 'fy'):
        assert lines[k].startswith('(300 (') and lines[k].endswith(f' {cells})(')
        vals = np.array([[float(x) for x in ln.split()] for ln in lines[k + 1:k + 1 + cells]])
        assert lines[k + 1 + cells] == '))'
        if name == 'uv':
            out['u'], out['v'] = vals[:, 0], vals[:, 1]
        else:
            out[name] = vals[:, 0]
        k += cells + 2
    return out


@pytest.mark.parametrize('case', CASES)
def test_case_ark_round_trip_is_byte_exact(case, tmp_path):
    src = GOLD / case / 'Case.ark'
    subprocess.run([runner(), 'rewrite-ark', src, tmp_path / 'Case.ark'], check=True)
    assert (tmp_path / 'Case.ark').read_bytes() == src.read_bytes()


@pytest.mark.parametrize('case', CASES)
@pytest.mark.parametrize('step', [0, 20])
def test_flowfield_writer_reproduces_the_reference_layout(case, step, tmp_path):
    name, text = golden_dat(case, step)
    (tmp_path / name).write_bytes(text)
    subprocess.run([runner(), 'rewrite-flowfield', tmp_path / name, tmp_path / 'out.dat'], check=True)
    assert (tmp_path / 'out.dat').read_bytes() == text


def test_case_ark_decodes_the_reference_constants():
    out = subprocess.run([runner(), 'show-config', GOLD / 'ac_ff' / 'Case.ark'], check=True, capture_output=True,
                         text=True).stdout.split()
    kv = dict(zip(out[0::2], out[1::2]))
    assert kv['model'] == '0' and kv['nx'] == '32' and kv['ny'] == '24' and kv['walls'] == '0'
    assert kv['init'] == '0' and float(kv['param']) == 7.0
    assert float(kv['Mu0']) == 0.02 and float(kv['Sigma']) == 1e-3 and float(kv['RhoV']) == 0.1
    assert kv['flux'] == '0'  # "CD = Flux Scheme"
    out = subprocess.run([runner(), 'show-config', GOLD / 'uw_ff' / 'Case.ark'], check=True, capture_output=True,
                         text=True).stdout.split()
    assert dict(zip(out[0::2], out[1::2]))['flux'] == '1'  # "UW = Flux Scheme"


@pytest.mark.parametrize('grad,flux', [('6points', '1'), ('LS', '2'), ('4points', '3')])
def test_case_ark_selects_the_uw_cell_gradient(tmp_path, grad, flux):
    """A 'cell gradient' entry picks the UW gradient the reference selects in its source
    (Grad_VS_6points / Grad_VS_LS / Grad_VS_4points)."""
    ark = tmp_path / 'Case.ark'
    ark.write_text((GOLD / 'uw_ff' / 'Case.ark').read_text() + f'{grad}    =    cell gradient\n')
    out = subprocess.run([runner(), 'show-config', ark], check=True, capture_output=True, text=True).stdout.split()
    assert dict(zip(out[0::2], out[1::2]))['flux'] == flux
    # the Rayleigh-Taylor box: walls from the mesh name; no case name, so an init entry is required
    r = subprocess.run([runner(), 'show-config', GOLD / 'hcz_rt' / 'Case.ark'], capture_output=True, text=True)
    assert r.returncode == 1 and "give an 'init' entry" in r.stderr


def test_flowfield_sections_hold_the_reference_fields_in_cell_order():
    """The golden FlowField of the AC_Drop case at step 20 against the CPU
    restatement (pinned to the reference): which field each section holds,
    and the cell order (cell (i, j) is line j*nx + i)."""
    from oracle.oracle import Oracle
    nx, ny = 32, 24
    o = Oracle('AC', nx, ny, False, 'ac_drop', Mu0=0.02, W=4.0, Sigma=1e-3, RhoL=1.0, RhoV=0.1, radius=7.0)
    o.step(20)
    _, text = golden_dat('ac_ff', 20)
    ff = parse_flowfield(text, nx * ny)
    for sec, fld in (('rho', 'rho'), ('u', 'u'), ('v', 'v'), ('p', 'p'), ('phi', 'phi'), ('tau', 'tauf'),
                     ('fx', 'fx'), ('fy', 'fy')):
        ref = o.get(fld).reshape(-1)
        # 12 significant digits in the file
        assert np.allclose(ff[sec], ref, rtol=2e-12, atol=1e-300), sec
    assert np.all(ff['T'] == float('3.333333333333e-01'))


GRID = {'ac_ff': (32, 24), 'uw_ff': (32, 24), 'hcz_rt': (16, 64), 'nee_rt': (16, 64)}


def golden_profiles(case: str) -> list[Path]:
    return sorted(GOLD.joinpath(case, 'Convergence').glob('*.dat'))


def test_golden_profiles_are_present():
    """Every case has MidX and MidY after the last step; Diag only where ny >= nx."""
    for case, (nx, ny) in GRID.items():
        kinds = sorted(f.name.split('_')[0] for f in golden_profiles(case))
        assert kinds == (['Diag', 'MidX', 'MidY'] if ny >= nx else ['MidX', 'MidY']), case


@pytest.mark.parametrize('case', CASES)
def test_profile_writer_reproduces_the_reference_layout(case, tmp_path):
    """Parse each golden MidX / MidY / Diag file and write it back: byte-identical
    (zone headers, the M_Phi title at the file's precision, coordinates, 4-space
    separators)."""
    nx, ny = GRID[case]
    for f in golden_profiles(case):
        kind = f.name.split('_')[0]
        subprocess.run([runner(), 'rewrite-profile', kind, str(nx), str(ny), f, tmp_path / f.name], check=True)
        assert (tmp_path / f.name).read_bytes() == f.read_bytes(), f.name


@pytest.mark.gpu
@pytest.mark.parametrize('case,extra', [('ac_ff', []),
                                        ('hcz_rt', ['--set', 'init=ac_rt', '--set', 'gravity=0.0001']),
                                        ('uw_ff', []),
                                        ('nee_rt', ['--set', 'init=ac_rt', '--set', 'gravity=0.0001',
                                                    '--set', 'wall scheme=NEE'])])
def test_driver_output_equals_the_reference_files(case, extra, tmp_path):
    """dugks_run on the reference's Case.ark, plain FP64 path: Case.ark, the
    FlowField files at steps 0 and 20 and the MidX / MidY / Diag profiles at step
    20 (thermoPressure included) are byte-identical to the reference's."""
    out = tmp_path / 'FlowField'
    subprocess.run([runner(), 'run', GOLD / case / 'Case.ark', '--out', out, '--steps', '20'] + extra, check=True,
                   capture_output=True)
    for step in (0, 20):
        name, text = golden_dat(case, step)
        assert (out / 'global' / name).read_bytes() == text, (case, step)
    for f in golden_profiles(case):
        assert (out / 'Convergence' / f.name).read_bytes() == f.read_bytes(), (case, f.name)


@pytest.mark.gpu
@pytest.mark.parametrize('case', ['ac_ff', 'uw_ff'])
def test_driver_drop_l2_equals_the_reference(case, tmp_path):
    """AC_Drop_L2Norm after 20 steps of the reference's AC_Drop case: the value
    dugks_run --l2 prints equals the reference's to the last bit."""
    out = tmp_path / 'FlowField'
    r = subprocess.run([runner(), 'run', GOLD / case / 'Case.ark', '--out', out, '--steps', '20', '--l2',
                        '--set', 'residual every=10'], check=True, capture_output=True, text=True)
    got = [ln.split()[1] for ln in r.stdout.splitlines() if ln.startswith('L2_phi ')]
    want = json.loads(GOLD.joinpath(case, 'l2.json').read_text())['L2_phi']
    assert got and float(got[0]) == float(want), (got, want)
    rows = next(out.joinpath('Convergence').glob('L2_uvp_mu*.dat')).read_text().splitlines()
    assert len(rows) == 2 and float(rows[-1].split()[1]) == float(f'{float(want):.8e}')


@pytest.mark.gpu
@pytest.mark.parametrize('case,extra', [('ac_ff', []), ('uw_ff', []),
                                        ('nee_rt', ['--set', 'init=ac_rt', '--set', 'gravity=0.0001',
                                                    '--set', 'wall scheme=NEE'])])
def test_driver_fp32_run_is_close_to_the_reference_files(case, extra, tmp_path):
    """FP32 storage through dugks_run against the reference's FlowField files at step 20
    (the AC_Drop case with the central and the upwind scheme, and the Rayleigh-Taylor box
    with NEE walls)."""
    out = tmp_path / 'FlowField'
    subprocess.run([runner(), 'run', GOLD / case / 'Case.ark', '--out', out, '--steps', '20', '--precision',
                    'fp32dev'] + extra, check=True, capture_output=True)
    name, text = golden_dat(case, 20)
    nx, ny = GRID[case]
    a = parse_flowfield((out / 'global' / name).read_bytes(), nx * ny)
    b = parse_flowfield(text, nx * ny)
    for k in ('rho', 'p', 'phi', 'tau', 'T'):
        assert np.max(np.abs(a[k] - b[k])) <= 1e-5 * np.max(np.abs(b[k])), k
    for k in ('fx', 'fy'):
        assert np.max(np.abs(a[k] - b[k])) <= 1e-3 * np.max(np.abs(b[k])), k
