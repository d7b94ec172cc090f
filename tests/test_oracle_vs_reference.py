"""Live pin of the oracle against freshly built reference binaries.

Runs only where the reference sources are mounted (the build container);
the committed fixtures cover the same ground everywhere else.
"""
import build_ref
import numpy as np
import pytest

from oracle.oracle import Oracle, read_dump
from variants import VARIANTS

pytestmark = pytest.mark.skipif(not build_ref.available(), reason='reference sources not mounted')


@pytest.mark.parametrize('name', ['ac_small', 'hcz_rt', 'pp_drop'])
def test_live_reference_bitexact(name, tmp_path):
    import build_ref
    build_ref.build(name)
    steps = 37
    out, _ = build_ref.run(name, steps, threads=4, dump=str(tmp_path / 'd.bin'))
    _, ref = read_dump(out)
    o = Oracle.from_variant(VARIANTS[name])
    o.step(steps)
    n = 0
    for k, r in ref.items():
        try:
            a = o.get(k)
        except KeyError:
            continue
        assert np.array_equal(a, r), k
        n += 1
    assert n > 10
