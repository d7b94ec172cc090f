"""Host side of the drop-in: Case.ark reader/writer, FlowField writer and the
dugks_run driver, against files written by the reference's own OutputCase and
Output_Flowfield (tests/golden/flowfield, made by make_flowfield_golden.py)."""
import gzip
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


@pytest.mark.gpu
@pytest.mark.parametrize('case,extra', [('ac_ff', []),
                                        ('hcz_rt', ['--set', 'init=ac_rt', '--set', 'gravity=0.0001']),
                                        ('uw_ff', []),
                                        ('nee_rt', ['--set', 'init=ac_rt', '--set', 'gravity=0.0001',
                                                    '--set', 'wall scheme=NEE'])])
def test_driver_output_equals_the_reference_files(case, extra, tmp_path):
    """dugks_run on the reference's Case.ark, plain FP64 path: Case.ark and the
    FlowField files at steps 0 and 20 are byte-identical to the reference's."""
    out = tmp_path / 'FlowField'
    subprocess.run([runner(), 'run', GOLD / case / 'Case.ark', '--out', out, '--steps', '20'] + extra, check=True,
                   capture_output=True)
    for step in (0, 20):
        name, text = golden_dat(case, step)
        assert (out / 'global' / name).read_bytes() == text, (case, step)


@pytest.mark.gpu
def test_driver_fp32_run_is_close_to_the_reference_files(tmp_path):
    out = tmp_path / 'FlowField'
    subprocess.run([runner(), 'run', GOLD / 'ac_ff' / 'Case.ark', '--out', out, '--steps', '20', '--precision',
                    'fp32dev'], check=True, capture_output=True)
    name, text = golden_dat('ac_ff', 20)
    a = parse_flowfield((out / 'global' / name).read_bytes(), 32 * 24)
    b = parse_flowfield(text, 32 * 24)
    for k in ('rho', 'p', 'phi', 'tau', 'T'):
        assert np.max(np.abs(a[k] - b[k])) <= 1e-5 * np.max(np.abs(b[k])), k
    for k in ('fx', 'fy'):
        assert np.max(np.abs(a[k] - b[k])) <= 1e-3 * np.max(np.abs(b[k])), k
