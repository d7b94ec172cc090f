"""CPU checks of the benchmark's analysis helpers."""
import numpy as np
import pytest

A = dict(abs=1e-5)  # the helper rounds to 5 decimals


def test_rt_fronts_of_a_flat_and_a_perturbed_interface():
    import bench
    nx, ny, c = 64, 256, 128
    phi = np.zeros((ny, nx))
    phi[c:, :] = 1.0  # heavy phase above row c
    f = bench.rt_fronts(phi, nx, c / nx)
    assert f['spike'] == pytest.approx(0.5 / nx, **A) and f['bubble'] == pytest.approx(-0.5 / nx, **A)
    assert f['mixing_zone'] == 0.0
    # a heavy finger 20 rows down in one column, a light bubble 10 rows up in another
    phi[c - 20:c, 5] = 1.0
    phi[c:c + 10, 40] = 0.0
    f = bench.rt_fronts(phi, nx, c / nx)
    assert f['spike'] == pytest.approx((c - 20 + 0.5 - c) / nx, **A)
    assert f['bubble'] == pytest.approx((c + 9 + 0.5 - c) / nx, **A)
    assert f['mixing_zone'] == pytest.approx(30 / nx, **A)  # 20 rows with mean 1/64, 10 with mean 63/64


def test_reference_arm_prints_the_contract_line():
    """bench.py --impl reference: W warm-up and K timed steps of the CPU restatement, one
    JSON line with the reference arm's keys (no GPU involved)."""
    import json
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    r = subprocess.run([sys.executable, str(root / 'bench.py'), '--impl', 'reference', '--steps', '2',
                        '--warmup', '3'], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d['impl'] == 'reference' and d['metric'] == 'MLUPS' and d['unit'] == 'MLUPS'
    assert d['steps'] == 2 and d['warmup'] == 3 and d['value'] > 0 and d['higher_is_better'] is True
    assert d['cpu_baseline']['kind'] == 'port' and d['cpu_baseline']['value'] == d['value']
    assert d['e2e'] == {'value': d['value'], 'unit': 'MLUPS', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}
