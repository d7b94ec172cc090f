"""Slab decomposition (dugks_slabs_*): the partition plan, its halo exchange
schedule across processes (gloo, CPU) and, on the GPU, partitioned runs equal
to the undivided case."""
import os
import socket

import numpy as np
import pytest

H = 2  # halo rows per side


def free_port() -> int:
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


@pytest.mark.parametrize('ny,walls,n', [(64, False, 1), (64, False, 3), (100, True, 3), (17, True, 2), (800, False, 7)])
def test_plan_covers_the_grid(ny, walls, n):
    from mpdugks_gb300 import capi
    row0, nrows, lo, hi = capi.slab_plan(ny, walls, n)
    assert row0[0] == 0 and sum(nrows) == ny
    assert all(row0[p] + nrows[p] == row0[p + 1] for p in range(n - 1))
    assert min(nrows) >= 8 and max(nrows) - min(nrows) <= 1
    for p in range(n):
        if walls:
            assert lo[p] == (p - 1 if p > 0 else -1) and hi[p] == (p + 1 if p < n - 1 else -1)
        else:
            assert lo[p] == (p - 1) % n and hi[p] == (p + 1) % n


def test_plan_rejects_too_many_partitions():
    from mpdugks_gb300 import capi
    with pytest.raises(capi.DugksError) as e:
        capi.slab_plan(20, False, 3)
    assert e.value.code == capi.DUGKS_EINVAL


# ---- the exchange schedule across processes (gloo): each rank owns a slab of a
# global array with two halo rows per side and executes the library's own halo
# schedule (dugks_slabs_schedule, the list the device exchange runs after every
# step): it sends the copies whose source it owns and receives those it is the
# destination of, tagged by their index in the schedule

def _exchange_rank(rank, world, port, ny, walls, fail_rank, q):
    import torch
    import torch.distributed as dist
    from datetime import timedelta
    from mpdugks_gb300 import capi
    try:
        os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
        dist.init_process_group('gloo', rank=rank, world_size=world, timeout=timedelta(seconds=5))
        row0, nrows, lo, hi = capi.slab_plan(ny, walls, world)
        copies = capi.slab_schedule(ny, walls, world)
        nx = 5
        glob = np.arange(ny * nx, dtype=np.float64).reshape(ny, nx) + 1.0
        r0, n = row0[rank], nrows[rank]
        mine = np.zeros((n + 2 * H, nx))
        mine[H:H + n] = glob[r0:r0 + n]
        if rank == fail_rank:
            raise RuntimeError('rank left before the exchange')
        reqs = []
        for tag, (src, srow, dst, drow, rows) in enumerate(copies):
            if src == rank:
                reqs.append(dist.isend(torch.from_numpy(mine[H + srow:H + srow + rows].copy()), dst, tag=tag))
        for tag, (src, srow, dst, drow, rows) in enumerate(copies):
            if dst == rank:
                t = torch.empty((rows, nx), dtype=torch.float64)
                dist.recv(t, src, tag=tag)
                mine[H + drow:H + drow + rows] = t.numpy()
        for r in reqs:
            r.wait()
        for k in range(-H, n + H):
            g = r0 + k
            if not walls:
                g %= ny
            if 0 <= g < ny and (k >= 0 or lo[rank] >= 0) and (k < n or hi[rank] >= 0):
                assert np.array_equal(mine[H + k], glob[g]), (rank, k)
        dist.destroy_process_group()
        q.put((rank, 'ok'))
    except Exception as e:  # reported to the parent
        q.put((rank, f'error: {type(e).__name__}: {e}'))


def _run_exchange(ny, walls, fail_rank=-1, world=2):
    import multiprocessing as mp
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_exchange_rank, args=(r, world, port, ny, walls, fail_rank, q))
             for r in range(world)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        if p.is_alive():
            p.kill()
    return out


@pytest.mark.parametrize('ny,walls,world', [(40, False, 2), (41, True, 2), (50, False, 3), (35, True, 4)])
def test_halo_exchange_schedule_across_ranks(ny, walls, world):
    out = _run_exchange(ny, walls, world=world)
    assert out == {r: 'ok' for r in range(world)}, out


@pytest.mark.parametrize('ny,walls,n', [(40, False, 2), (41, True, 2), (64, False, 4), (33, True, 3)])
def test_schedule_fills_every_halo_row_once(ny, walls, n):
    """Every halo row next to a neighbour is written by exactly one copy, from the
    neighbour's matching boundary rows; wall sides get no copy."""
    from mpdugks_gb300 import capi
    row0, nrows, lo, hi = capi.slab_plan(ny, walls, n)
    seen = {}
    for src, srow, dst, drow, rows in capi.slab_schedule(ny, walls, n):
        assert rows == H
        for k in range(rows):
            key = (dst, drow + k)
            assert key not in seen
            seen[key] = (src, srow + k)
    want = {}
    for p in range(n):
        if lo[p] >= 0:
            for k in range(H):
                want[(p, -H + k)] = (lo[p], nrows[lo[p]] - H + k)
        if hi[p] >= 0:
            for k in range(H):
                want[(p, nrows[p] + k)] = (hi[p], k)
    assert seen == want


def test_a_rank_that_leaves_is_reported_not_waited_for():
    out = _run_exchange(40, False, fail_rank=1)
    assert out[1].startswith('error') and 'left before' in out[1]
    assert out[0].startswith('error'), out[0]  # the peer's receive fails within its timeout


# ---- the device data path

@pytest.mark.gpu
@pytest.mark.parametrize('model,walls,nx,ny,n,init,params,kw', [
    ('AC', False, 64, 96, 3, 'ac_drop_inside', [20.0], dict(Mu0=0.01, M_Phi=0.05, W=4.0, Sigma=1e-3, RhoL=1.0,
                                                             RhoV=0.1)),
    ('AC', False, 40, 24, 1, 'ac_drop_inside', [8.0], dict(Mu0=0.01, W=4.0, Sigma=1e-3, RhoL=1.0, RhoV=0.1)),
    ('HCZ', True, 48, 100, 3, 'ac_rt', [1.0, 0.1, 1e-4], dict(Mu0=0.01, M_Phi=0.05, W=4.0, Sigma=1e-4, RhoL=3.0,
                                                               RhoV=1.0, Gy=1e-4)),
    ('HCZ', False, 50, 300, 2, 'ac_drop_inside', [15.0], dict(Mu0=0.02, W=4.0, Sigma=1e-2, RhoL=10.0, RhoV=1.0)),
    # large enough for the undivided case to take the streaming kernel with TMA row loads,
    # against partitions whose rows (halo rows included) are loaded per lane
    ('HCZ', True, 1120, 1664, 2, 'ac_rt', [0.75, 0.1, 1e-4], dict(Mu0=0.01, M_Phi=0.05, W=4.0, Sigma=1e-4,
                                                                   RhoL=3.0, RhoV=1.0, Gy=1e-4)),
])
def test_partitioned_run_equals_the_undivided_case(model, walls, nx, ny, n, init, params, kw):
    from mpdugks_gb300 import capi
    steps = 33
    sl = capi.Slabs(capi.make_case(model, 'fp32dev', **kw), nx, ny, walls, n)
    sl.init(init, params, seed=5)
    gc = capi.GpuCase(capi.make_case(model, 'fp32dev', **kw), nx, ny, walls)
    gc.init(init, params, seed=5)
    red = []
    for _ in range(2):  # the second residual is the change over `steps` steps
        sl.step(steps)
        gc.step(steps)
        red.append((sl.reduce(), gc.reduce()))
    a = sl.fields()
    sl.close()
    for k in ('rho', 'u', 'v', 'phi', 'p'):
        assert np.array_equal(a[k], gc.get(k)), k
    # the same sums as the undivided case, added in another order
    for rs, rg in red:
        assert rs.steps == rg.steps
        assert abs(rs.sum_rho - rg.sum_rho) <= 1e-13 * abs(rg.sum_rho)
        assert abs(rs.sum_phi - rg.sum_phi) <= 1e-12 * abs(rg.sum_phi)
        assert abs(rs.residual - rg.residual) <= 1e-9 * rg.residual
