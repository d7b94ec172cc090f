"""A rewriting the exact FP64 step relies on, checked on the CPU against IEEE arithmetic
(a C restatement of the device function): a quotient by a shared divisor from its
correctly rounded reciprocal plus one fused multiply-add correction (Markstein).  It
must give the IEEE quotient bit for bit, or the exact path stops matching the reference."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


def run_check(tmp_path, source: str, n: int):
    gcc = shutil.which('gcc')
    if gcc is None:
        pytest.skip('gcc not available')
    exe = tmp_path / Path(source).stem
    subprocess.run([gcc, '-O2', '-ffp-contract=off', '-o', str(exe), str(HERE / source), '-lm'], check=True)
    r = subprocess.run([str(exe), str(n)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip().endswith('0 mismatches'), r.stdout


def test_shared_reciprocal_quotient_is_the_ieee_quotient(tmp_path):
    run_check(tmp_path, 'qdiv_check.c', 20_000_000)
