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
