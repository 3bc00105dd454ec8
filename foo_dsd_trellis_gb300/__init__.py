"""foo_dsd_trellis_gb300 — GB300-native PCM/DSD -> DSD conversion hot path.

The compute lives in libdsdgpu.so (CUDA kernels for sm_103a behind the C ABI
of include/dsdgpu.h).  This package holds the Python side of that boundary:
the ctypes binding (_lib), the NTF table (ntf) and host mirrors of the
reference's interfaces (sdm, ...).
"""
from . import ntf  # noqa: F401

__all__ = ["ntf"]
