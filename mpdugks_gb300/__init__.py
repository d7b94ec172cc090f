"""GB300-native DUGKS time-step library (sm_103a CUDA behind a C ABI).

``capi`` binds libdugks_gpu.so (include/dugks_gpu.h) with ctypes; ``build``
compiles it (and the ``dugks_run`` driver) in-tree for sm_103a.  The CUDA
kernels and the C ABI live in ``csrc/``; the host driver that mirrors the
reference's main() + DUGKS2DSolver (Case.ark reader/writer, FlowField and
line-profile writers, .cas mesh reader) lives in ``host/``.
"""
from . import build  # noqa: F401

__all__ = ['build']
