"""Host-side mirror of the reference's PreCorr SDM interface over libdsdgpu.

`PreCorr` follows precorr_context_init / precorr_process_block /
precorr_context_reset (include/precorr.h:49-61, src/precorr.c:198-287) for a
bank of channels sharing one NTF and one trained table; the reference's own
GPU entry point (gpu_precorr_process, include/gpu_compute.h:140-144) runs one
channel per call, this one runs them all in one launch.  Outputs are 0/1
decision bytes (the reference writes +-1 floats).  Device buffers are torch
CUDA tensors; every computation runs in libdsdgpu's kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib


class PreCorr:
    def __init__(self, order: int, a, g, state_limit: float = 0.0, num_channels: int = 1,
                 device: int = 0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.dsdgpu_create(device, C.byref(h))
        if rc != _lib.OK:
            raise _lib.DsdGpuError(rc, "dsdgpu_create failed")
        self.h = h
        self.device = device
        aa = np.zeros(10, np.float64)
        gg = np.zeros(10, np.float64)
        aa[:order] = np.asarray(a, np.float64)[:order]
        gg[:order] = np.asarray(g, np.float64)[:order]
        _lib.check(self.h, self.L.dsdgpu_precorr_setup(
            self.h, order, aa.ctypes.data, gg.ctypes.data, float(state_limit), num_channels))
        self.order = order
        self.num_channels = num_channels

    def close(self):
        if getattr(self, "h", None):
            self.L.dsdgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def table(self) -> np.ndarray:
        """The trained correction table, float32 [256 histories][8 phases]."""
        t = np.zeros(256 * 8, np.float32)
        _lib.check(self.h, self.L.dsdgpu_precorr_table(self.h, t.ctypes.data))
        return t.reshape(256, 8)

    def reset(self) -> None:
        _lib.check(self.h, self.L.dsdgpu_precorr_reset(self.h))

    def process_block(self, x: torch.Tensor, first: int = 0) -> torch.Tensor:
        """x: [nch, count] float64 on this device -> uint8 decisions [nch, count]."""
        x = x.to(torch.float64).contiguous()
        if x.dim() == 1:
            x = x.unsqueeze(0)
        nch, count = x.shape
        out = torch.empty((nch, max(count, 1)), dtype=torch.uint8, device=x.device)
        torch.cuda.current_stream().synchronize()
        _lib.check(self.h, self.L.dsdgpu_precorr_process(
            self.h, first, nch, x.data_ptr(), count, count, out.data_ptr(), out.shape[1]))
        return out[:, :count]
