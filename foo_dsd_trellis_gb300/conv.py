"""UPOLS convolution at the SDM rate over libdsdgpu (dsdgpu_conv_*): the
reference's room-correction convolver (src/convolution.c:355-405,
src/gpu_cuda.c:3432-3492), FP32, whole chunks per call, history carried."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib


def setup(L, h, ir: np.ndarray, partition: int = 4096) -> None:
    """Install per-channel IRs (float32 [nch, taps]) on context h."""
    ir = np.ascontiguousarray(np.atleast_2d(ir), np.float32)
    _lib.check(h, L.dsdgpu_conv_setup(h, ir.ctypes.data_as(C.c_void_p), ir.shape[1], ir.shape[0],
                                      partition))


class Convolver:
    def __init__(self, ir: np.ndarray, partition: int = 4096, device: int = 0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.dsdgpu_create(device, C.byref(h))
        if rc != _lib.OK:
            raise _lib.DsdGpuError(rc, "dsdgpu_create failed")
        self.h = h
        setup(self.L, h, ir, partition)
        self.nch = int(np.atleast_2d(ir).shape[0])

    def process(self, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """x: float64 [nch, n] CUDA -> convolved float64 [nch, n] (history carried)."""
        x = x.to(torch.float64).contiguous()
        if out is None:
            out = torch.empty_like(x)
        torch.cuda.current_stream().synchronize()
        _lib.check(self.h, self.L.dsdgpu_conv_process(self.h, x.shape[0], C.c_void_p(x.data_ptr()),
                                                      x.stride(0), x.shape[1],
                                                      C.c_void_p(out.data_ptr()), out.stride(0)))
        return out

    def reset(self) -> None:
        _lib.check(self.h, self.L.dsdgpu_conv_reset(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.L.dsdgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
