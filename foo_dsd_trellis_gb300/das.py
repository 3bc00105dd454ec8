"""Host-side mirror of the reference's DAS chunk processing over libdsdgpu.

`DasChannels` owns one persistent trellis SDM context per channel (the
reference's s->channels[ch].sdm) and runs chunks through segment-parallel
SDM + Density-Aligned Stitching on the GPU (src/dsp_plugin.c:1283-2762).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib

FULL_PARALLEL = _lib.DAS_FULL_PARALLEL
SEG0_FIRST = _lib.DAS_SEG0_FIRST


class DasChannels:
    def __init__(self, order: int, a, g, depth: int, cands: int, lat: int,
                 state_limit: float = 0.0, num_channels: int = 2, device: int = 0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.dsdgpu_create(device, C.byref(h))
        if rc != _lib.OK:
            raise _lib.DsdGpuError(rc, "dsdgpu_create failed")
        self.h = h
        p = _lib.SdmParams()
        p.order = order
        for i in range(order):
            p.a[i] = float(a[i])
            p.g[i] = float(g[i])
        p.depth, p.cands, p.lat, p.state_limit = depth, cands, lat, float(state_limit)
        _lib.check(self.h, self.L.dsdgpu_sdm_setup(self.h, C.byref(p), num_channels))
        self.nch = num_channels
        self.lat = lat
        self.device = device

    def set_select(self, mode: int) -> None:
        _lib.check(self.h, self.L.dsdgpu_set_option(self.h, _lib.OPT_SDM_SELECT, mode))

    def last_sdm_kernel(self) -> str:
        return _lib.last_sdm_kernel(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.L.dsdgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def process_chunk(self, fir: torch.Tensor, seg_len: int = 0, nsegs: int = 0,
                      seed_mode: int = FULL_PARALLEL, reposition: bool = True,
                      out: torch.Tensor | None = None):
        """fir: [nch, count] float64 CUDA.  Returns (decisions [nch, n] uint8, seams)."""
        fir = fir.to(torch.float64).contiguous()
        nch, count = fir.shape
        if out is None:
            out = torch.empty((nch, count), dtype=torch.uint8, device=fir.device)
        dp = _lib.DasParams(seg_len, nsegs, seed_mode, int(reposition))
        maxs = max(1, count // seg_len if seg_len > 0 else nsegs)
        seams = (C.c_int * maxs)()
        n = C.c_size_t()
        torch.cuda.current_stream().synchronize()
        _lib.check(self.h, self.L.dsdgpu_das_process(
            self.h, C.byref(dp), nch, C.c_void_p(fir.data_ptr()), count, count,
            C.c_void_p(out.data_ptr()), out.stride(0), C.byref(n), seams, maxs))
        return out[:, : n.value], list(seams)
