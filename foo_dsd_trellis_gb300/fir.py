"""Host-side mirror of the reference's FIR chain interface over libdsdgpu.

`FirChain` stands in for fir_chain_init_ex + fir_chain_process_d plus the
engine's glue on the rate-conversion path (boxcar pre-smooth, gain ramp, tanh
soft clip; reference src/engine.c:608-717): one object per channel group,
history carried across blocks like the reference's delay lines.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib


class FirChain:
    def __init__(self, fs_in: int, fs_out: int, boxcar_taps: int = 8, soft_clip: bool = True,
                 num_channels: int = 1, device: int = 0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.dsdgpu_create(device, C.byref(h))
        if rc != _lib.OK:
            raise _lib.DsdGpuError(rc, "dsdgpu_create failed")
        self.h = h
        p = _lib.FirParams()
        p.fs_in, p.fs_out, p.boxcar_taps, p.soft_clip = fs_in, fs_out, boxcar_taps, int(soft_clip)
        _lib.check(self.h, self.L.dsdgpu_fir_setup(self.h, C.byref(p), num_channels))
        self.ratio = fs_out // fs_in
        self.num_channels = num_channels
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.L.dsdgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self):
        _lib.check(self.h, self.L.dsdgpu_fir_reset(self.h))

    def process(self, pcm: torch.Tensor, gain_start: float = 1.0, gain_end: float = 1.0,
                first: int = 0, out: torch.Tensor | None = None) -> torch.Tensor:
        """pcm: [nch, n] float32 CUDA -> [nch, n * ratio] float64 CUDA."""
        pcm = pcm.to(torch.float32).contiguous()
        if pcm.dim() == 1:
            pcm = pcm.unsqueeze(0)
        nch, n = pcm.shape
        if out is None:
            out = torch.empty((nch, n * self.ratio), dtype=torch.float64, device=pcm.device)
        oc = C.c_size_t()
        torch.cuda.current_stream().synchronize()
        _lib.check(self.h, self.L.dsdgpu_fir_process(
            self.h, first, nch, C.c_void_p(pcm.data_ptr()), n, n, C.c_void_p(out.data_ptr()),
            out.stride(0), float(gain_start), float(gain_end), C.byref(oc)))
        return out
