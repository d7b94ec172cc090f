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
    # under 8 rows: the batch lane's tile kernel, in the same model group as streaming items
    (lambda: ac_case(), 40, 6, False, 'ac_drop_inside', [2.0], 45),
    # pseudopotential FP32 cases: solo lanes, concurrently
    (lambda: pp_case('PP16'), 40, 40, False, 'scmp_drop', [], 80),
    (lambda: pp_case('PP9'), 48, 48, False, 'pp_noise', [0.2, 0.01], 90),
    # FP32 storage with the UW flux scheme and with NEE walls: solo lanes
    (lambda: ac_case(scheme='UW'), 64, 48, False, 'ac_drop_inside', [10.0], 70),
    (lambda: nee_case(), 32, 64, True, 'ac_rt', [1.0, 0.1, 1e-4], 55),
]


def nee_case():
    from mpdugks_gb300 import capi
    return capi.make_case('HCZ', 'fp32dev', Mu0=0.01, M_Phi=0.05, W=4.0, Sigma=1e-4, RhoL=3.0, RhoV=1.0,
                          Gy=1e-4, wall='NEE')


def pp_case(model, precision='fp32dev'):
    from mpdugks_gb300 import capi
    return capi.make_case(model, precision)


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


@pytest.mark.parametrize('item', [-2, -1], ids=['fp32_uw', 'fp32_nee'])
def test_solo_lane_fp32_variants_match_the_plain_path(item):
    """FP32 cases the batched kernels do not take (UW flux scheme, NEE walls) run in a solo
    lane and equal the same case stepped through its own handle."""
    from mpdugks_gb300 import capi
    f, nx, ny, w, init, params, n = MIX[item]
    srv = capi.Server(chunk_steps=16)
    r = run(srv, [MIX[item], MIX[0]])[0]
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
    # ragged: a last strip of 25 columns, a last segment of 27 rows
    (lambda: rt_case(), 1117, 1531, True, 'ac_rt', [0.7, 0.1, 1e-4], 23),
    # small: the single-case step runs the tile kernel, the server the batched streaming kernel
    (lambda: rt_case(), 64, 128, True, 'ac_rt', [1.0, 0.1, 1e-4], 29),
    # under 8 rows: the tile kernel on both sides (batched in the server)
    (lambda: ac_case(), 40, 6, False, 'ac_drop_inside', [2.0], 31),
])
def test_streaming_kernel_equals_the_tile_kernel(item):
    """A case solved by the server (batched streaming kernel k_streamb32; the batched
    tile kernel for cases under 8 rows) against the same case stepped alone (the
    streaming kernel k_stream32, with TMA row loads, where the grid has more strip
    segments than resident warps; the tile kernel otherwise).  With walls and
    without, they agree bit for bit."""
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


# ---- stopping rule and FlowField output

GOLD = __import__('pathlib').Path(__file__).resolve().parent / 'golden' / 'flowfield'


def golden_case(precision):
    """The reference's own AC_Drop 32x24 case of tests/golden/flowfield/ac_ff."""
    from mpdugks_gb300 import capi
    return capi.make_case('AC', precision, Mu0=0.02, M_Phi=0.1, W=4.0, Sigma=1e-3, RhoL=1.0, RhoV=0.1)


def golden_file(step):
    import gzip
    f = next((GOLD / 'ac_ff').glob(f'step{step}Ma*.dat.gz'))
    return f.name[:-3], gzip.decompress(f.read_bytes())


def parse_flowfield(text, cells):
    lines = text.decode().splitlines()
    out, k = {}, 0
    for name in ('rho', 'uv', 'p', 'T', 'phi', 'tau', 'fx', 'fy'):
        vals = np.array([[float(x) for x in ln.split()] for ln in lines[k + 1:k + 1 + cells]])
        if name == 'uv':
            out['u'], out['v'] = vals[:, 0], vals[:, 1]
        else:
            out[name] = vals[:, 0]
        k += cells + 2
    return out


def test_flowfield_files_equal_the_reference_files(tmp_path):
    """The plain FP64 path in a solo lane, with snapshots every 10 steps: the
    files at steps 0 and 20 are byte-identical to the reference's own
    Output_Flowfield files (a snapshot in between does not disturb the run)."""
    from mpdugks_gb300 import capi
    srv = capi.Server()
    cid = srv.submit(golden_case('fp64'), 32, 24, False, 'ac_drop', [7.0], nsteps=20, snapshot_every=10,
                     out_dir=str(tmp_path))
    st = srv.wait(cid, 120.0)
    stats = srv.stats()
    srv.close()
    assert st.state == 2 and st.files == 3 and stats.files_written == 3
    for step in (0, 20):
        name, text = golden_file(step)
        assert (tmp_path / name).read_bytes() == text, step
    assert (tmp_path / 'step10Ma0_Car32_CFL0.5_T5.dat').exists()


def test_batched_flowfield_files_are_close_to_the_reference_files(tmp_path):
    """The same case in FP32 storage, batched with another case: the file at
    step 20 agrees with the reference's to 1e-5 (rho, p, phi, tau)."""
    from mpdugks_gb300 import capi
    srv = capi.Server(chunk_steps=8)
    cid = srv.submit(golden_case('fp32dev'), 32, 24, False, 'ac_drop', [7.0], nsteps=20, snapshot_every=12,
                     out_dir=str(tmp_path))
    other = srv.submit(ac_case(), 64, 64, False, 'ac_drop_inside', [12.0], nsteps=60)
    st = srv.wait(cid, 120.0)
    assert srv.wait(other, 120.0).state == 2
    srv.close()
    assert st.state == 2 and st.batched == 1 and st.files == 3
    name, text = golden_file(20)
    a = parse_flowfield((tmp_path / name).read_bytes(), 32 * 24)
    b = parse_flowfield(text, 32 * 24)
    for k in ('rho', 'p', 'phi', 'tau', 'T'):
        assert np.max(np.abs(a[k] - b[k])) <= 1e-5 * np.max(np.abs(b[k])), k
    assert (tmp_path / 'step12Ma0_Car32_CFL0.5_T6.dat').exists()


@pytest.mark.parametrize('precision', ['fp32dev', 'fp64'])
def test_case_stops_at_the_first_check_below_the_tolerance(precision):
    """Residual every 50 steps as the reference's Update_Residual; the case stops
    at the first check at or below the tolerance, with the fields of that step."""
    from mpdugks_gb300 import capi
    every, checks = 50, 6
    gc = capi.GpuCase(ac_case(precision), 64, 64, False)
    gc.init('ac_drop_inside', [12.0], seed=7)
    res, fields = [], []
    for _ in range(checks):
        gc.step(every)
        res.append(gc.reduce().residual)
        fields.append({k: gc.get(k) for k in FIELDS})
    tol = res[3]
    stop = next(k for k, r in enumerate(res) if r <= tol)
    srv = capi.Server(chunk_steps=16)
    cid = srv.submit(ac_case(precision), 64, 64, False, 'ac_drop_inside', [12.0], seed=7, nsteps=100000,
                     residual_tol=tol, check_every=every)
    other = srv.submit(ac_case(precision), 48, 48, False, 'ac_drop_inside', [10.0], nsteps=130)
    st = srv.wait(cid, 300.0)
    assert srv.wait(other, 300.0).state == 2
    r = srv.result(cid)
    stats = srv.stats()
    srv.close()
    assert st.state == 2 and st.stop_reason == 1, (st.state, st.stop_reason)
    assert st.steps_done == every * (stop + 1) and st.residual == res[stop]
    assert stats.converged == 1
    for k in FIELDS:
        assert np.array_equal(r[k], fields[stop][k]), k


def test_diverging_cases_are_stopped_and_reported():
    """A state that overflows (phi noise of 1e200) fails at the first check,
    batched and in a solo lane, while a healthy case in the mix completes."""
    from mpdugks_gb300 import capi
    srv = capi.Server(chunk_steps=16)
    bad = [srv.submit(rt_case(p), 32, 64, True, 'ac_rt', [1.0, 0.1, 1e200], nsteps=5000, check_every=40)
           for p in ('fp32dev', 'fp64')]
    good = srv.submit(ac_case(), 48, 48, False, 'ac_drop_inside', [10.0], nsteps=100)
    sts = [srv.wait(c, 300.0) for c in bad]
    assert srv.wait(good, 300.0).state == 2
    stats = srv.stats()
    srv.close()
    for st in sts:
        assert st.state == 4 and st.stop_reason == 2 and st.steps_done == 40, (st.state, st.stop_reason,
                                                                             st.steps_done)
    assert stats.diverged == 2 and stats.completed == 1
