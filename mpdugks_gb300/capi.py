"""ctypes binding of libdugks_gpu.so (the C ABI in include/dugks_gpu.h).

The library is built in-tree by ``mpdugks_gb300.build``; loading fails loudly
when it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import build as _build

DUGKS_OK, DUGKS_EINVAL, DUGKS_ENOMEM, DUGKS_ECUDA, DUGKS_ETIMEOUT, DUGKS_ENAN = range(6)
STATUS_NAMES = {0: 'DUGKS_OK', 1: 'DUGKS_EINVAL', 2: 'DUGKS_ENOMEM', 3: 'DUGKS_ECUDA', 4: 'DUGKS_ETIMEOUT',
                5: 'DUGKS_ENAN'}
MODELS = {'AC': 0, 'HCZ': 1, 'PP9': 2, 'PP16': 3}
PRECISION = {'fp64': 0, 'fp32dev': 1, 'fp64fma': 2, 'fp64fused': 3}
FIELDS = ['rho', 'u', 'v', 'p', 'phi', 'tauf', 'phix', 'phiy', 'rhox', 'rhoy', 'fx', 'fy', 'prevphiu', 'prevphiv',
          'psi', 'scg']
INIT_KINDS = {'ac_drop': 0, 'ac_drop_inside': 1, 'ac_rt': 2, 'scmp_drop': 3, 'pp_noise': 4}


class DugksError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f'{STATUS_NAMES.get(code, code)}: {msg}')
        self.code = code


class CaseT(C.Structure):
    _fields_ = [('model', C.c_int), ('precision', C.c_int), ('Mu0', C.c_double), ('M_Phi', C.c_double),
                ('W', C.c_double), ('Sigma', C.c_double), ('RhoL', C.c_double), ('RhoV', C.c_double),
                ('Gy', C.c_double), ('Tr', C.c_double), ('aCS', C.c_double), ('Tc_CS', C.c_double),
                ('d2v16_c', C.c_double), ('flux_scheme', C.c_int), ('wall_scheme', C.c_int)]


class GridT(C.Structure):
    _fields_ = [('nx', C.c_int), ('ny', C.c_int), ('y_walls', C.c_int)]


class ReductionsT(C.Structure):
    _fields_ = [('sum_rho', C.c_double), ('sum_phi', C.c_double), ('residual', C.c_double),
                ('steps', C.c_int64)]


class HaloCopyT(C.Structure):
    _fields_ = [('src', C.c_int), ('src_row', C.c_int), ('dst', C.c_int), ('dst_row', C.c_int), ('rows', C.c_int)]


class SrvConfigT(C.Structure):
    _fields_ = [('max_bytes', C.c_size_t), ('chunk_steps', C.c_int), ('solo_lanes', C.c_int),
                ('reserved', C.c_int * 5)]


class SrvRequestT(C.Structure):
    _fields_ = [('cs', CaseT), ('grid', GridT), ('init_kind', C.c_int), ('nparams', C.c_int),
                ('params', C.POINTER(C.c_double)), ('seed', C.c_uint64), ('nsteps', C.c_int64),
                ('residual_tol', C.c_double), ('check_every', C.c_int), ('snapshot_every', C.c_int),
                ('out_dir', C.c_char_p)]


class SrvStatusT(C.Structure):
    _fields_ = [('state', C.c_int), ('batched', C.c_int), ('nsteps', C.c_int64), ('steps_done', C.c_int64),
                ('bytes', C.c_size_t), ('t_submit', C.c_double), ('t_start', C.c_double), ('t_done', C.c_double),
                ('stop_reason', C.c_int), ('files', C.c_int), ('residual', C.c_double)]


class SrvStatsT(C.Structure):
    _fields_ = [('submitted', C.c_int64), ('completed', C.c_int64), ('cancelled', C.c_int64), ('failed', C.c_int64),
                ('cell_updates', C.c_int64), ('chunks', C.c_int64), ('graphs_captured', C.c_int64),
                ('launches', C.c_int64), ('max_resident', C.c_int), ('bytes_in_use', C.c_size_t),
                ('bytes_peak', C.c_size_t), ('max_bytes', C.c_size_t), ('busy_s', C.c_double),
                ('converged', C.c_int64), ('diverged', C.c_int64), ('files_written', C.c_int64),
                ('solo_steps', C.c_int64)]


SRV_STATES = {0: 'queued', 1: 'running', 2: 'done', 3: 'cancelled', 4: 'failed'}
SRV_STOPS = {0: 'none', 1: 'converged', 2: 'diverged'}

# every symbol declared in include/dugks_gpu.h, with its ctypes signature
SIGNATURES = {
    'dugks_gpu_create': (C.c_int, [C.POINTER(CaseT), C.POINTER(GridT), C.POINTER(C.c_void_p)]),
    'dugks_gpu_nq': (C.c_int, [C.c_void_p]),
    'dugks_gpu_upload': (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    'dugks_gpu_init': (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_int, C.c_uint64]),
    'dugks_gpu_step': (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    'dugks_gpu_step_profiled': (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_double),
                                          C.POINTER(C.c_int)]),
    'dugks_gpu_reduce': (C.c_int, [C.c_void_p, C.POINTER(ReductionsT)]),
    'dugks_gpu_download': (C.c_int, [C.c_void_p] + [C.c_void_p] * 5),
    'dugks_gpu_get_field': (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    'dugks_gpu_drop_l2': (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    'dugks_gpu_thermo_pressure': (C.c_int, [C.c_void_p, C.c_void_p]),
    'dugks_gpu_set_field': (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    'dugks_gpu_get_dist': (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    'dugks_gpu_check_finite': (C.c_int, [C.c_void_p]),
    'dugks_gpu_last_error': (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    'dugks_gpu_launch_count': (C.c_int64, [C.c_void_p]),
    'dugks_gpu_destroy': (C.c_int, [C.c_void_p]),
    'dugks_gpu_checkpoint_bytes': (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t)]),
    'dugks_gpu_step_count': (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    'dugks_gpu_checkpoint': (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    'dugks_gpu_restore': (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    'dugks_gpu_step_noalloc': (C.c_int, [C.POINTER(CaseT), C.POINTER(GridT), C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_int, C.c_void_p]),
    'dugks_srv_create': (C.c_int, [C.POINTER(SrvConfigT), C.POINTER(C.c_void_p)]),
    'dugks_srv_submit': (C.c_int, [C.c_void_p, C.POINTER(CaseT), C.POINTER(GridT), C.c_int, C.POINTER(C.c_double),
                                   C.c_int, C.c_uint64, C.c_int64, C.POINTER(C.c_int64)]),
    'dugks_srv_submit_request': (C.c_int, [C.c_void_p, C.POINTER(SrvRequestT), C.POINTER(C.c_int64)]),
    'dugks_srv_poll': (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(SrvStatusT)]),
    'dugks_srv_wait': (C.c_int, [C.c_void_p, C.c_int64, C.c_double, C.POINTER(SrvStatusT)]),
    'dugks_srv_result': (C.c_int, [C.c_void_p, C.c_int64] + [C.c_void_p] * 5),
    'dugks_srv_release': (C.c_int, [C.c_void_p, C.c_int64]),
    'dugks_srv_cancel': (C.c_int, [C.c_void_p, C.c_int64]),
    'dugks_srv_stats': (C.c_int, [C.c_void_p, C.POINTER(SrvStatsT)]),
    'dugks_srv_last_error': (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    'dugks_srv_destroy': (C.c_int, [C.c_void_p]),
    'dugks_slabs_plan': (C.c_int, [C.c_int, C.c_int, C.c_int] + [C.POINTER(C.c_int)] * 4),
    'dugks_slabs_create': (C.c_int, [C.POINTER(CaseT), C.POINTER(GridT), C.c_int, C.POINTER(C.c_int),
                                     C.POINTER(C.c_void_p)]),
    'dugks_slabs_init': (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_int, C.c_uint64]),
    'dugks_slabs_step': (C.c_int, [C.c_void_p, C.c_int]),
    'dugks_slabs_schedule': (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(HaloCopyT), C.c_int,
                                       C.POINTER(C.c_int)]),
    'dugks_slabs_reduce': (C.c_int, [C.c_void_p, C.POINTER(ReductionsT)]),
    'dugks_slabs_download': (C.c_int, [C.c_void_p] + [C.c_void_p] * 5),
    'dugks_slabs_launch_count': (C.c_int64, [C.c_void_p]),
    'dugks_slabs_destroy': (C.c_int, [C.c_void_p]),
}

_lib = None


def library_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load libdugks_gpu.so; raise if it is not built (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        if not build_if_missing:
            raise RuntimeError(f'{path} is not built; run `python -m mpdugks_gb300.build` '
                               '(the DUGKS kernels have no CPU fallback)')
        _build.build()
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


FLUX_SCHEMES = {'CD': 0, 'UW': 1, 'UW_LS': 2, 'UW_4P': 3}  # dugks_flux_scheme
WALL_SCHEMES = {'BB': 0, 'NEE': 1}


def make_case(model: str, precision: str = 'fp64', *, Mu0=0.1, M_Phi=0.1, W=5.0, Sigma=1e-2, RhoL=10.0,
              RhoV=1.0, Gy=0.0, Tr=0.85, aCS=1.0, Tc_CS=0.0943, d2v16_c=1.2, scheme='CD', wall='BB') -> CaseT:
    return CaseT(MODELS[model], PRECISION[precision], Mu0, M_Phi, W, Sigma, RhoL, RhoV, Gy, Tr, aCS, Tc_CS,
                 d2v16_c, FLUX_SCHEMES[scheme], WALL_SCHEMES[wall])


class GpuCase:
    """One resident case on the GPU, driven through the C ABI."""

    def __init__(self, case: CaseT, nx: int, ny: int, y_walls: bool = False):
        self.lib = load()
        self.nx, self.ny = nx, ny
        self.case = case
        self.grid = GridT(nx, ny, int(y_walls))
        h = C.c_void_p()
        rc = self.lib.dugks_gpu_create(C.byref(case), C.byref(self.grid), C.byref(h))
        if rc != DUGKS_OK:
            buf = C.create_string_buffer(512)
            self.lib.dugks_gpu_last_error(None, buf, 512)
            raise DugksError(rc, buf.value.decode())
        self.h = h
        self.Q = self.lib.dugks_gpu_nq(h)

    def _check(self, rc: int) -> None:
        if rc != DUGKS_OK:
            buf = C.create_string_buffer(512)
            self.lib.dugks_gpu_last_error(self.h, buf, 512)
            raise DugksError(rc, buf.value.decode())

    def close(self) -> None:
        if getattr(self, 'h', None):
            self.lib.dugks_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init(self, kind: str, params=(), seed: int = 12345) -> None:
        arr = (C.c_double * max(1, len(params)))(*params)
        self._check(self.lib.dugks_gpu_init(self.h, INIT_KINDS[kind], arr, len(params), seed))

    def upload(self, f: np.ndarray, hdist: np.ndarray | None, aux: np.ndarray) -> None:
        f = np.ascontiguousarray(f, dtype=np.float64)
        aux = np.ascontiguousarray(aux, dtype=np.float64)
        hp = None
        if hdist is not None:
            hdist = np.ascontiguousarray(hdist, dtype=np.float64)
            hp = hdist.ctypes.data
        self._check(self.lib.dugks_gpu_upload(self.h, f.ctypes.data, hp, aux.ctypes.data))

    def step(self, n: int = 1, stream: int | None = None) -> None:
        self._check(self.lib.dugks_gpu_step(self.h, n, stream))

    def step_profiled(self, n: int, stream: int | None = None) -> list[float]:
        ms = (C.c_double * 4)()
        nph = C.c_int()
        self._check(self.lib.dugks_gpu_step_profiled(self.h, n, stream, ms, C.byref(nph)))
        return [ms[k] for k in range(nph.value)]

    def reduce(self) -> ReductionsT:
        r = ReductionsT()
        self._check(self.lib.dugks_gpu_reduce(self.h, C.byref(r)))
        return r

    def drop_l2(self) -> float:
        """AC_Drop_L2Norm (Ark/Cpp/Output.cpp:226-238) of the current phase field."""
        v = C.c_double()
        self._check(self.lib.dugks_gpu_drop_l2(self.h, C.byref(v)))
        return v.value

    def thermo_pressure(self) -> np.ndarray:
        """thermoPressure (Ark/Cpp/Output.cpp:146-163) of every cell, [ny][nx]."""
        out = np.empty((self.ny, self.nx), dtype=np.float64)
        self._check(self.lib.dugks_gpu_thermo_pressure(self.h, out.ctypes.data))
        return out

    def get(self, name: str) -> np.ndarray:
        out = np.empty((self.ny, self.nx), dtype=np.float64)
        self._check(self.lib.dugks_gpu_get_field(self.h, FIELDS.index(name), out.ctypes.data))
        return out

    def set(self, name: str, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.ny, self.nx)
        self._check(self.lib.dugks_gpu_set_field(self.h, FIELDS.index(name), a.ctypes.data))

    def dist(self, which: str = 'f') -> np.ndarray:
        out = np.empty((self.Q, self.ny, self.nx), dtype=np.float64)
        self._check(self.lib.dugks_gpu_get_dist(self.h, 0 if which == 'f' else 1, out.ctypes.data))
        return out

    def checkpoint(self) -> np.ndarray:
        """The whole device state as a byte array (dugks_gpu_checkpoint)."""
        n = C.c_size_t()
        self._check(self.lib.dugks_gpu_checkpoint_bytes(self.h, C.byref(n)))
        buf = np.empty(n.value, dtype=np.uint8)
        self._check(self.lib.dugks_gpu_checkpoint(self.h, buf.ctypes.data, n.value))
        return buf

    def restore(self, buf: np.ndarray) -> None:
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        self._check(self.lib.dugks_gpu_restore(self.h, buf.ctypes.data, buf.nbytes))

    def check_finite(self) -> int:
        return self.lib.dugks_gpu_check_finite(self.h)

    @property
    def launches(self) -> int:
        return self.lib.dugks_gpu_launch_count(self.h)


class Server:
    """A serving loop on the GPU (dugks_srv_*): submit cases, poll or wait, read results."""

    def __init__(self, max_bytes: int = 0, chunk_steps: int = 0, solo_lanes: int = 0):
        self.lib = load()
        cfg = SrvConfigT(max_bytes, chunk_steps, solo_lanes)
        h = C.c_void_p()
        rc = self.lib.dugks_srv_create(C.byref(cfg), C.byref(h))
        if rc != DUGKS_OK:
            raise DugksError(rc, 'dugks_srv_create failed')
        self.s = h
        self.shapes: dict[int, tuple[int, int]] = {}

    def _check(self, rc: int) -> None:
        if rc != DUGKS_OK:
            buf = C.create_string_buffer(512)
            self.lib.dugks_srv_last_error(self.s, buf, 512)
            raise DugksError(rc, buf.value.decode())

    def submit(self, case: CaseT, nx: int, ny: int, y_walls: bool, init: str, params=(), seed: int = 12345,
               nsteps: int = 100, residual_tol: float = 0.0, check_every: int = 0, snapshot_every: int = 0,
               out_dir: str | None = None) -> int:
        """Queue a case: nsteps steps at most; every check_every steps (0: 1000) it stops
        converged once the residual is <= residual_tol (0: never) and fails when not
        finite; with out_dir, FlowField files at step 0, every snapshot_every steps
        and at the end."""
        arr = (C.c_double * max(1, len(params)))(*params)
        cid = C.c_int64()
        rq = SrvRequestT(case, GridT(nx, ny, int(y_walls)), INIT_KINDS[init], len(params), arr, seed, nsteps,
                         residual_tol, check_every, snapshot_every,
                         None if out_dir is None else os.fsencode(out_dir))
        self._check(self.lib.dugks_srv_submit_request(self.s, C.byref(rq), C.byref(cid)))
        self.shapes[cid.value] = (ny, nx)
        return cid.value

    def poll(self, cid: int) -> SrvStatusT:
        st = SrvStatusT()
        self._check(self.lib.dugks_srv_poll(self.s, cid, C.byref(st)))
        return st

    def wait(self, cid: int, timeout: float = -1.0) -> SrvStatusT:
        st = SrvStatusT()
        self._check(self.lib.dugks_srv_wait(self.s, cid, timeout, C.byref(st)))
        return st

    def result(self, cid: int) -> dict[str, np.ndarray]:
        ny, nx = self.shapes[cid]
        out = {k: np.empty((ny, nx), dtype=np.float64) for k in ('rho', 'u', 'v', 'phi', 'p')}
        self._check(self.lib.dugks_srv_result(self.s, cid, *[out[k].ctypes.data for k in ('rho', 'u', 'v', 'phi',
                                                                                             'p')]))
        return out

    def release(self, cid: int) -> None:
        self._check(self.lib.dugks_srv_release(self.s, cid))
        self.shapes.pop(cid, None)

    def cancel(self, cid: int) -> None:
        self._check(self.lib.dugks_srv_cancel(self.s, cid))

    def stats(self) -> SrvStatsT:
        st = SrvStatsT()
        self._check(self.lib.dugks_srv_stats(self.s, C.byref(st)))
        return st

    def close(self) -> None:
        if getattr(self, 's', None):
            self.lib.dugks_srv_destroy(self.s)
            self.s = None

    def __del__(self):
        self.close()


def slab_plan(ny: int, y_walls: bool, nparts: int):
    """Host-only partition plan: (row0, nrows, lo, hi) lists (lo/hi -1: a wall)."""
    lib = load()
    arrs = [(C.c_int * nparts)() for _ in range(4)]
    rc = lib.dugks_slabs_plan(ny, int(y_walls), nparts, *arrs)
    if rc != DUGKS_OK:
        buf = C.create_string_buffer(512)
        lib.dugks_gpu_last_error(None, buf, 512)
        raise DugksError(rc, buf.value.decode())
    return tuple([list(a) for a in arrs])


def slab_schedule(ny: int, y_walls: bool, nparts: int) -> list[tuple[int, int, int, int, int]]:
    """Host-only halo exchange schedule: (src, src_row, dst, dst_row, rows) per copy, in
    the order the device exchange issues them (local rows; negative = lower halo)."""
    lib = load()
    n = C.c_int()
    rc = lib.dugks_slabs_schedule(ny, int(y_walls), nparts, None, 0, C.byref(n))
    if rc == DUGKS_OK:
        out = (HaloCopyT * max(1, n.value))()
        rc = lib.dugks_slabs_schedule(ny, int(y_walls), nparts, out, n.value, C.byref(n))
    if rc != DUGKS_OK:
        buf = C.create_string_buffer(512)
        lib.dugks_gpu_last_error(None, buf, 512)
        raise DugksError(rc, buf.value.decode())
    return [(c.src, c.src_row, c.dst, c.dst_row, c.rows) for c in out[:n.value]]


class Slabs:
    """One FP32-storage case split along y into partitions with halo exchange (dugks_slabs_*)."""

    def __init__(self, case: CaseT, nx: int, ny: int, y_walls: bool, nparts: int, devices=None):
        self.lib = load()
        self.nx, self.ny = nx, ny
        grid = GridT(nx, ny, int(y_walls))
        dev = (C.c_int * nparts)(*devices) if devices else None
        h = C.c_void_p()
        self._check(self.lib.dugks_slabs_create(C.byref(case), C.byref(grid), nparts, dev, C.byref(h)))
        self.h = h

    def _check(self, rc: int) -> None:
        if rc != DUGKS_OK:
            buf = C.create_string_buffer(512)
            self.lib.dugks_gpu_last_error(None, buf, 512)
            raise DugksError(rc, buf.value.decode())

    def init(self, kind: str, params=(), seed: int = 12345) -> None:
        arr = (C.c_double * max(1, len(params)))(*params)
        self._check(self.lib.dugks_slabs_init(self.h, INIT_KINDS[kind], arr, len(params), seed))

    def step(self, n: int = 1) -> None:
        self._check(self.lib.dugks_slabs_step(self.h, n))

    def reduce(self) -> ReductionsT:
        r = ReductionsT()
        self._check(self.lib.dugks_slabs_reduce(self.h, C.byref(r)))
        return r

    def fields(self) -> dict[str, np.ndarray]:
        out = {k: np.empty((self.ny, self.nx), dtype=np.float64) for k in ('rho', 'u', 'v', 'phi', 'p')}
        self._check(self.lib.dugks_slabs_download(self.h, *[out[k].ctypes.data for k in ('rho', 'u', 'v', 'phi',
                                                                                           'p')]))
        return out

    def close(self) -> None:
        if getattr(self, 'h', None):
            self.lib.dugks_slabs_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
