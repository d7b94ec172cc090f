"""Host buffers through the C ABI: pinned, mapped host memory (read and written in place by
kernels over the host link) and pageable memory (copy-engine staging) give the same state
and the same downloaded fields, bit for bit."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host_state(capi, nx, ny):
    src = capi.GpuCase(capi.make_case('HCZ', 'fp64', Gy=1e-4, RhoL=3.0, RhoV=1.0, Sigma=1e-4, W=4.0), nx, ny, True)
    src.init('ac_rt')
    src.step(3)
    f, h = src.dist('f'), src.dist('h')
    aux = np.stack([src.get(k) for k in capi.FIELDS])
    return f, h, aux


@pytest.mark.parametrize('precision', ['fp32dev', 'fp64fused'])
def test_pinned_and_pageable_host_buffers_agree(precision):
    torch = pytest.importorskip('torch')
    from mpdugks_gb300 import capi
    nx, ny = 96, 40
    f, h, aux = _host_state(capi, nx, ny)
    kw = dict(Gy=1e-4, RhoL=3.0, RhoV=1.0, Sigma=1e-4, W=4.0)
    a = capi.GpuCase(capi.make_case('HCZ', precision, **kw), nx, ny, True)
    b = capi.GpuCase(capi.make_case('HCZ', precision, **kw), nx, ny, True)
    a.upload(f, h, aux)  # pageable numpy arrays
    pf, ph, pa = (torch.from_numpy(x.copy()).pin_memory() for x in (f, h, aux))
    b._check(b.lib.dugks_gpu_upload(b.h, pf.data_ptr(), ph.data_ptr(), pa.data_ptr()))
    a.step(25)
    b.step(25)
    outs_a = [np.empty((ny, nx)) for _ in range(5)]
    outs_b = [torch.empty((ny, nx), dtype=torch.float64).pin_memory() for _ in range(5)]
    a._check(a.lib.dugks_gpu_download(a.h, *[C.c_void_p(o.ctypes.data) for o in outs_a]))
    b._check(b.lib.dugks_gpu_download(b.h, *[C.c_void_p(o.data_ptr()) for o in outs_b]))
    for k, (x, y) in enumerate(zip(outs_a, outs_b)):
        assert np.array_equal(x, y.numpy()), k
    assert np.isfinite(outs_a[0]).all() and float(np.abs(outs_a[0]).max()) > 0
