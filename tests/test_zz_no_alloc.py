"""The no-allocation step entry point against the handle-based one.

dugks_gpu_step_noalloc serves callers that may not allocate device memory
(a host with a fixed memory budget or its own pool, a plugin inside another
runtime, a loop that must not allocate once running): the caller owns the
state buffers and the step's scratch lives in a fixed device array inside the
library.  Here the caller's buffers are torch tensors; the entry point itself
allocates nothing.  Its results must equal those of dugks_gpu_step through a
handle, to the same bar as the other FP64 tests -- bit for bit for the
reference-exact precision -- on two calls in a row (the second call reuses the
scratch the first one left behind).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from variants import VARIANTS  # noqa: E402

MODEL = {'D2Q9AC': 'AC', 'D2Q9HCZ': 'HCZ'}
KEYS = ('Mu0', 'M_Phi', 'W', 'Sigma', 'RhoL', 'RhoV', 'Gy')


def _handle_case(v):
    from mpdugks_gb300 import capi
    c = v['consts']
    case = capi.make_case(MODEL[v['model']], 'fp64', **{k: c[k] for k in KEYS if k in c})
    gc = capi.GpuCase(case, v['nx'], v['ny'], v['walls'])
    if v['init'] == 'ac_rt':
        gc.init('ac_rt')
    else:
        gc.init(v['init'], [c.get('radius', -1.0)])
    return case, gc


def _state(gc):
    from mpdugks_gb300 import capi
    return gc.dist('f'), gc.dist('h'), np.stack([gc.get(k) for k in capi.FIELDS])


@pytest.mark.parametrize('name', ['hcz_rt', 'ac_small'])
def test_noalloc_matches_handle_two_calls(name):
    import torch
    from mpdugks_gb300 import capi
    v = VARIANTS[name]
    case, gc = _handle_case(v)
    f0, h0, a0 = _state(gc)
    dev = torch.device('cuda', torch.cuda.current_device())
    df = torch.from_numpy(f0.copy()).to(dev)
    dh = torch.from_numpy(h0.copy()).to(dev)
    da = torch.from_numpy(a0.copy()).to(dev)
    grid = capi.GridT(v['nx'], v['ny'], int(v['walls']))
    lib = capi.load()
    stream = torch.cuda.current_stream().cuda_stream
    n = 37
    for call in range(2):
        rc = lib.dugks_gpu_step_noalloc(C.byref(case), C.byref(grid), df.data_ptr(), dh.data_ptr(),
                                        da.data_ptr(), n, stream)
        assert rc == capi.DUGKS_OK
        torch.cuda.synchronize()
        gc.step(n)
        f1, h1, a1 = _state(gc)  # reading fields completes the handle's last step the same way
        assert np.array_equal(df.cpu().numpy(), f1), f'{name} call {call}: f differs'
        assert np.array_equal(dh.cpu().numpy(), h1), f'{name} call {call}: h differs'
        got = da.cpu().numpy()
        for k, fld in enumerate(capi.FIELDS):
            assert np.array_equal(got[k], a1[k]), f'{name} call {call}: field {fld} differs'


def test_noalloc_rejects_grids_beyond_the_scratch():
    import torch
    from mpdugks_gb300 import capi
    lib = capi.load()
    case = capi.make_case('AC', 'fp64')
    grid = capi.GridT(128, 64, 0)  # 8192 cells > 4096: rejected before any device work
    buf_dev = torch.zeros(8, dtype=torch.float64, device='cuda')
    p = buf_dev.data_ptr()
    rc = lib.dugks_gpu_step_noalloc(C.byref(case), C.byref(grid), p, p, p, 1, None)
    assert rc == capi.DUGKS_EINVAL
    buf = C.create_string_buffer(256)
    lib.dugks_gpu_last_error(None, buf, 256)
    assert b'4096' in buf.value


def test_noalloc_inside_a_captured_graph():
    """One direct call, then the same call captured into a CUDA graph on a side
    stream and replayed: the capture reuses the scratch address the direct call
    looked up, and the replay equals a second direct call bit for bit."""
    import torch
    from mpdugks_gb300 import capi
    v = VARIANTS['ac_small']
    case, gc = _handle_case(v)
    f0, h0, a0 = _state(gc)
    dev = torch.device('cuda', torch.cuda.current_device())
    df = torch.from_numpy(f0.copy()).to(dev)
    dh = torch.from_numpy(h0.copy()).to(dev)
    da = torch.from_numpy(a0.copy()).to(dev)
    grid = capi.GridT(v['nx'], v['ny'], int(v['walls']))
    lib = capi.load()
    n = 11
    rc = lib.dugks_gpu_step_noalloc(C.byref(case), C.byref(grid), df.data_ptr(), dh.data_ptr(), da.data_ptr(), n,
                                    torch.cuda.current_stream().cuda_stream)
    assert rc == capi.DUGKS_OK
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side, capture_error_mode='thread_local'):
            rc = lib.dugks_gpu_step_noalloc(C.byref(case), C.byref(grid), df.data_ptr(), dh.data_ptr(),
                                            da.data_ptr(), n, side.cuda_stream)
    assert rc == capi.DUGKS_OK
    g.replay()
    torch.cuda.synchronize()
    gc.step(2 * n)
    f1, h1, a1 = _state(gc)
    assert np.array_equal(df.cpu().numpy(), f1)
    assert np.array_equal(dh.cpu().numpy(), h1)
    got = da.cpu().numpy()
    for k, fld in enumerate(capi.FIELDS):
        assert np.array_equal(got[k], a1[k]), fld
