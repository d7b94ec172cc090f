import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / 'oracle' / 'ref'))

GOLDEN = ROOT / 'tests' / 'golden'


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (the GB300 parity and kernel tests)')


def pytest_collection_modifyitems(config, items):
    # keep the no-allocation entry point's test file last, whatever the selection
    items.sort(key=lambda it: 1 if 'test_zz_' in it.nodeid else 0)


@pytest.fixture(scope='session')
def golden():
    import json
    import numpy as np
    meta = json.loads((GOLDEN / 'golden_meta.json').read_text())

    def load(name):
        d = np.load(GOLDEN / f'{name}.npz')
        out = {}
        for k in d.files:
            fld, st = k.split('@')
            out.setdefault(int(st), {})[fld] = d[k]
        return out
    return meta, load


def rel_err(a, b):
    """max-norm relative error max|a-b| / max|b| (0 when both are 0)."""
    import numpy as np
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = float(np.max(np.abs(b)))
    num = float(np.max(np.abs(a - b)))
    if den == 0.0:
        return num
    return num / den
