"""Serving loop (dugks_srv_*): continuous batching, admission by footprint,
cancellation, and results that do not depend on the other cases."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ('rho', 'u', 'v', 'phi', 'p')


def ac_case(precision='fp32dev', **kw):
    from mpdugks_gb300 import capi
    base = dict(Mu0=0.01, M_Phi=0.05, W=4.0, Sigma=1e-3, RhoL=1.0, RhoV=0.1)
    base.update(kw)
    return capi.make_case('AC', precision, **base)


def rt_case(precision='fp32dev'):
    from mpdugks_gb300 import capi
    return capi.make_case('HCZ', precision, Mu0=0.01, M_Phi=0.05, W=4.0, Sigma=1e-4, RhoL=3.0, RhoV=1.0,
                          Gy=1e-4)


# (case factory, nx, ny, walls, init, params, nsteps)
MIX = [
    (lambda: ac_case(), 96, 96, False, 'ac_drop_inside', [20.0], 150),
    (lambda: rt_case(), 64, 128, True, 'ac_rt', [1.0, 0.1, 1e-4], 97),
    (lambda: ac_case(Sigma=5e-3, RhoV=0.5), 130, 70, False, 'ac_drop', [15.0], 61),
    (lambda: ac_case('fp64'), 48, 48, False, 'ac_drop_inside', [10.0], 40),
    (lambda: ac_case(RhoV=0.02), 200, 40, False, 'ac_drop_inside', [12.0], 203),
]


def run(server, items):
    ids = [server.submit(f(), nx, ny, w, init, params, seed=7, nsteps=n) for f, nx, ny, w, init, params, n in items]
    out = []
    for cid in ids:
        st = server.wait(cid, 300.0)
        assert st.state == 2, (cid, st.state)
        out.append(server.result(cid))
    return out


def test_results_identical_alone_and_in_the_mix():
    from mpdugks_gb300 import capi
    alone = []
    srv = capi.Server(chunk_steps=16)
    for item in MIX:
        alone.append(run(srv, [item])[0])
    srv.close()
    srv = capi.Server(chunk_steps=16)
    mixed = run(srv, MIX)
    st = srv.stats()
    srv.close()
    assert st.completed == len(MIX) and st.failed == 0
    assert st.max_resident >= 2  # the cases really ran together
    for k, (a, b) in enumerate(zip(alone, mixed)):
        for f in FIELDS:
            assert np.array_equal(a[f], b[f]), (k, f)


def test_batched_case_matches_the_single_case_kernel():
    """A batched FP32 case and the same case stepped through its own handle."""
    from mpdugks_gb300 import capi
    f, nx, ny, w, init, params, n = MIX[1]
    srv = capi.Server(chunk_steps=16)
    r = run(srv, [MIX[1], MIX[0]])[0]
    srv.close()
    gc = capi.GpuCase(f(), nx, ny, w)
    gc.init(init, params, seed=7)
    gc.step(n)
    for k in FIELDS:
        assert np.array_equal(r[k], gc.get(k)), k


def test_solo_lane_fp64_matches_the_plain_path():
    from mpdugks_gb300 import capi
    f, nx, ny, w, init, params, n = MIX[3]
    srv = capi.Server(chunk_steps=16)
    r = run(srv, [MIX[3], MIX[0]])[0]
    srv.close()
    gc = capi.GpuCase(f(), nx, ny, w)
    gc.init(init, params, seed=7)
    gc.step(n)
    for k in FIELDS:
        assert np.array_equal(r[k], gc.get(k)), k


def test_admission_respects_the_byte_budget():
    from mpdugks_gb300 import capi, build  # noqa: F401
    probe = capi.Server()
    one = probe.poll(probe.submit(ac_case(), 128, 128, False, 'ac_drop_inside', [25.0], nsteps=1)).bytes
    probe.close()
    srv = capi.Server(max_bytes=int(2.5 * one), chunk_steps=8)
    items = [(lambda: ac_case(), 128, 128, False, 'ac_drop_inside', [25.0], 40 + 7 * k) for k in range(6)]
    run(srv, items)
    st = srv.stats()
    srv.close()
    assert st.completed == 6
    assert st.max_resident == 2
    assert st.bytes_peak <= st.max_bytes


def test_cancel_and_oversized_submit():
    from mpdugks_gb300 import capi
    srv = capi.Server(max_bytes=64 << 20, chunk_steps=8)
    long_id = srv.submit(ac_case(), 128, 128, False, 'ac_drop_inside', [25.0], nsteps=10 ** 7)
    short_id = srv.submit(ac_case(), 64, 64, False, 'ac_drop_inside', [12.0], nsteps=24)
    assert srv.wait(short_id, 120.0).state == 2
    srv.cancel(long_id)
    st = srv.wait(long_id, 120.0)
    assert st.state == 3
    with pytest.raises(capi.DugksError) as ei:
        srv.submit(ac_case(), 4096, 4096, False, 'ac_drop_inside', [25.0], nsteps=1)
    assert ei.value.code == capi.DUGKS_ENOMEM
    srv.close()


@pytest.mark.parametrize('item', [
    (lambda: ac_case(), 560, 3300, False, 'ac_drop_inside', [200.0], 37),
    (lambda: rt_case(), 560, 3300, True, 'ac_rt', [3.0, 0.1, 1e-4], 41),
])
def test_streaming_kernel_equals_the_tile_kernel(item):
    """Single-case FP32 steps on a grid of more strip segments than resident warps
    run the streaming kernel (warps marching 28-column strips through row
    segments); the server runs the tile kernel.  With walls and without, they
    agree bit for bit."""
    from mpdugks_gb300 import capi
    f, nx, ny, w, init, params, n = item
    srv = capi.Server(chunk_steps=16)
    r = run(srv, [item])[0]
    srv.close()
    gc = capi.GpuCase(f(), nx, ny, w)
    gc.init(init, params, seed=7)
    gc.step(n)
    for k in FIELDS:
        assert np.array_equal(r[k], gc.get(k)), k
