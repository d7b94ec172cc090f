"""The numpy restatement of the output quantities (oracle/outputs.py) pinned to
the reference's own output: thermoPressure against the TP zones of the golden
MidX / MidY / Diag files, and AC_Drop_L2Norm against the golden l2.json, both
from the golden FlowField fields of the same step (printed with 13 significant
digits, which bounds the agreement).  The walled cases' ghost rows extrapolate
the step's final phase field here, the step's starting one in the reference; the
two differ by far less than the tolerance next to walls where phi is flat."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import outputs as O
from test_host import GOLD, golden_dat, parse_flowfield

# nx, ny, W, Sigma, RhoL, RhoV, walls (oracle/ref/variants.py)
CASES = {'ac_ff': (32, 24, 4.0, 1e-3, 1.0, 0.1, False), 'uw_ff': (32, 24, 4.0, 1e-3, 1.0, 0.1, False),
         'hcz_rt': (16, 64, 4.0, 1e-4, 3.0, 1.0, True), 'nee_rt': (16, 64, 4.0, 1e-4, 3.0, 1.0, True)}


def zone(path: Path, name: str) -> np.ndarray:
    lines = path.read_text().splitlines()
    k = next(i for i, ln in enumerate(lines) if ln.startswith(f'zone T = {name}_M'))
    out = []
    for ln in lines[k + 1:]:
        if ln.startswith('variables'):
            break
        out.append(float(ln.split()[1]))
    return np.array(out)


def fields(case):
    nx, ny, W, S, RL, RV, walls = CASES[case]
    _, text = golden_dat(case, 20)
    ff = parse_flowfield(text, nx * ny)
    return nx, ny, walls, O.constants(W, S, RL, RV), ff['phi'].reshape(ny, nx), ff['p'].reshape(ny, nx)


@pytest.mark.parametrize('case', list(CASES))
def test_thermo_pressure_matches_the_reference_profiles(case):
    nx, ny, walls, k, phi, p = fields(case)
    tp = O.thermo_pressure(phi, p, k, walls)
    conv = GOLD / case / 'Convergence'
    checked = 0
    for f in sorted(conv.glob('*.dat')):
        g = zone(f, 'TP')
        if f.name.startswith('MidX'):
            mine = tp[:, nx // 2 - 1]
        elif f.name.startswith('MidY'):
            mine = tp[ny // 2 - 1, :]
        else:
            mine = tp[nx - 1 - np.arange(nx), np.arange(nx)]
        assert mine.shape == g.shape
        # TP carries kappa phi lap(phi): the 13-digit inputs give ~1e-12 of max|TP|;
        # Diag prints 9 significant digits
        tol = 1e-8 if f.name.startswith('Diag') else 2e-12
        assert np.max(np.abs(mine - g)) <= tol * max(1.0, np.max(np.abs(g))), f.name
        checked += 1
    assert checked >= 2


@pytest.mark.parametrize('case', ['ac_ff', 'uw_ff'])
def test_drop_l2_matches_the_reference(case):
    nx, ny, walls, k, phi, p = fields(case)
    want = float(json.loads((GOLD / case / 'l2.json').read_text())['L2_phi'])
    got = O.drop_l2(phi, 7.0, k)  # the variants' AC_Drop radius
    assert abs(got - want) <= 1e-9 * want, (got, want)
