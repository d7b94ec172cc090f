"""The FP64 step divides by a shared divisor through its correctly rounded reciprocal
and one fused multiply-add correction (Markstein); the result must be the IEEE
quotient bit for bit, or the exact path stops matching the reference."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


def test_shared_reciprocal_quotient_is_the_ieee_quotient(tmp_path):
    gcc = shutil.which('gcc')
    if gcc is None:
        pytest.skip('gcc not available')
    exe = tmp_path / 'qdiv_check'
    subprocess.run([gcc, '-O2', '-ffp-contract=off', '-o', str(exe), str(HERE / 'qdiv_check.c'), '-lm'], check=True)
    r = subprocess.run([str(exe), '20000000'], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip().endswith('0 mismatches'), r.stdout
