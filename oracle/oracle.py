"""ctypes front end of the CPU restatement -- TEST INFRASTRUCTURE ONLY.

Used by tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg as the checker; the product path never imports it.
"""
from __future__ import annotations

import ctypes as C
import struct
from pathlib import Path

import numpy as np

from . import build_oracle

MODELS = {'AC': 0, 'HCZ': 1, 'PP9': 2, 'PP16': 3}
INITS = {'ac_drop': 0, 'ac_drop_inside': 1, 'ac_rt': 2, 'scmp_drop': 3, 'pp_noise': 4}
REF_MODEL = {'D2Q9AC': 'AC', 'D2Q9HCZ': 'HCZ', 'D2Q9PP': 'PP9', 'D2V16PP': 'PP16'}


class _Inputs(C.Structure):
    _fields_ = [('model', C.c_int), ('nx', C.c_int), ('ny', C.c_int), ('y_walls', C.c_int),
                ('gravity', C.c_int), ('init', C.c_int),
                ('Mu0', C.c_double), ('M_Phi', C.c_double), ('W', C.c_double), ('Sigma', C.c_double),
                ('RhoL', C.c_double), ('RhoV', C.c_double), ('Gy', C.c_double), ('radius', C.c_double),
                ('Tr', C.c_double), ('aCS', C.c_double), ('Tc_CS', C.c_double), ('PP_RhoL', C.c_double),
                ('PP_RhoV', C.c_double), ('PP_radius', C.c_double), ('noise_rho0', C.c_double),
                ('noise_amp', C.c_double), ('seed', C.c_uint64), ('d2v16_c', C.c_double), ('uw', C.c_int),
                ('nee', C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(str(path))
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(_Inputs)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_step.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.orc_get.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p]
        L.orc_get.restype = C.c_int
        L.orc_set.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p]
        L.orc_set.restype = C.c_int
        L.orc_const.argtypes = [C.c_void_p, C.c_char_p]
        L.orc_const.restype = C.c_double
        L.orc_nq.argtypes = [C.c_void_p]
        L.orc_sums.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_steps_done.argtypes = [C.c_void_p]
        L.orc_steps_done.restype = C.c_long
        L.orc_velocities.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_velocities.restype = C.c_int
        L.orc_d2v16_equilibrium.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_void_p]
        L.orc_d2v16_equilibrium.restype = C.c_int
        _lib = L
    return _lib


DEFAULTS = dict(Mu0=0.1, M_Phi=0.1, W=5.0, Sigma=1e-2, RhoL=10.0, RhoV=1.0, Gy=0.0, radius=-1.0,
                Tr=0.85, aCS=1.0, Tc_CS=0.0943, PP_RhoL=2.4806e-1, PP_RhoV=4.5435e-2, PP_radius=-1.0,
                noise_rho0=0.2, noise_amp=0.01, seed=12345, d2v16_c=1.2, uw=0, nee=0)


# flux scheme of a variant -> orc_inputs.uw (the C ABI's dugks_flux_scheme values)
UW_CODE = {'CD': 0, 'UW': 1, 'UW_LS': 2, 'UW_4P': 3}


class Oracle:
    """One CPU-restatement solver instance."""

    def __init__(self, model: str, nx: int, ny: int, walls: bool = False, init: str = 'ac_drop', **consts):
        p = dict(DEFAULTS)
        for k, v in consts.items():
            if k == 'radius_frac':
                continue
            if k not in p:
                raise KeyError(k)
            p[k] = v
        self.inputs = _Inputs(model=MODELS[model], nx=nx, ny=ny, y_walls=int(walls),
                              gravity=int(consts.get('Gy', 0.0) != 0.0), init=INITS[init], **p)
        self.nx, self.ny = nx, ny
        self._h = lib().orc_create(C.byref(self.inputs))
        if not self._h:
            raise ValueError('orc_create failed')
        self.Q = lib().orc_nq(self._h)

    @classmethod
    def from_variant(cls, v: dict) -> 'Oracle':
        return cls(REF_MODEL[v['model']], v['nx'], v['ny'], v['walls'], v['init'], **v['consts'],
                   uw=UW_CODE[v.get('scheme', 'CD')], nee=int(v.get('wall', 'BB') == 'NEE'))

    def __del__(self):
        h = getattr(self, '_h', None)
        if h:
            lib().orc_destroy(h)
            self._h = None

    def step(self, n: int = 1, threads: int = 0) -> None:
        lib().orc_step(self._h, n, threads)

    @property
    def steps_done(self) -> int:
        return lib().orc_steps_done(self._h)

    def velocities(self):
        """(xi_u, xi_v, |xi|^2 + eta^2) of the model's discrete velocities."""
        a = [np.empty(self.Q) for _ in range(3)]
        lib().orc_velocities(self._h, *[x.ctypes.data for x in a])
        return tuple(a)

    def d2v16_equilibrium(self, rho: float, u: float, v: float) -> np.ndarray:
        eq = np.empty(16)
        if lib().orc_d2v16_equilibrium(self._h, rho, u, v, eq.ctypes.data) != 0:
            raise ValueError('not a D2V16 model')
        return eq

    def get(self, name: str) -> np.ndarray:
        out = np.empty((self.ny, self.nx), dtype=np.float64)
        if lib().orc_get(self._h, name.encode(), out.ctypes.data) != 0:
            raise KeyError(name)
        return out

    def set(self, name: str, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.ny, self.nx)
        if lib().orc_set(self._h, name.encode(), a.ctypes.data) != 0:
            raise KeyError(name)

    def const(self, name: str) -> float:
        return lib().orc_const(self._h, name.encode())

    def sums(self):
        a, b = C.c_double(), C.c_double()
        lib().orc_sums(self._h, C.byref(a), C.byref(b))
        return a.value, b.value

    def dists(self, which: str = 'f') -> np.ndarray:
        return np.stack([self.get(f'{which}{q}') for q in range(self.Q)])


def read_dump(path) -> tuple[int, dict]:
    """Read a binary dump written by oracle/ref/ref_driver.cpp."""
    raw = Path(path).read_bytes()
    magic, nx, ny, nf = struct.unpack_from('<4i', raw, 0)
    assert magic == 0x44554753, 'bad dump magic'
    (step,) = struct.unpack_from('<q', raw, 16)
    off = 24
    names = []
    for _ in range(nf):
        names.append(raw[off:off + 16].split(b'\0', 1)[0].decode())
        off += 16
    data = np.frombuffer(raw, dtype='<f8', offset=off).reshape(nf, ny, nx)
    return step, {n: data[k].copy() for k, n in enumerate(names)}
