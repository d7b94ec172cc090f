"""GB300-native DUGKS time-step library (sm_103a CUDA behind a C ABI).

``capi`` binds libdugks_gpu.so (include/dugks_gpu.h); ``solver`` is the host
loop that mirrors the reference's DUGKS2DSolver; ``casefile`` reads and writes
the reference's Case.ark key/value layout and FlowField output.
"""
from . import build  # noqa: F401

__all__ = ['build']
