"""Host-side mirror of the reference's DSD packers over libdsdgpu:
dop_pack_i24 (with the plugin's channel interleave) and bits_pack
(reference src/dop.c:114-184)."""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib


class Packer:
    def __init__(self, device: int = 0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.dsdgpu_create(device, C.byref(h))
        if rc != _lib.OK:
            raise _lib.DsdGpuError(rc, "dsdgpu_create failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.dsdgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def dop(self, bits: torch.Tensor, phase: int = 0):
        """bits [nch, n] uint8 CUDA -> ([n // 16, nch, 3] uint8 CUDA, next phase)."""
        bits = bits.contiguous()
        nch, n = bits.shape
        out = torch.empty((max(n // 16, 1), nch, 3), dtype=torch.uint8, device=bits.device)
        ph = C.c_int()
        torch.cuda.current_stream().synchronize()
        _lib.check(self.h, self.L.dsdgpu_pack_dop(self.h, nch, C.c_void_p(bits.data_ptr()),
                                                  bits.stride(0), n, C.c_void_p(out.data_ptr()),
                                                  phase, C.byref(ph)))
        return out[: n // 16], ph.value

    def native(self, bits: torch.Tensor) -> torch.Tensor:
        """bits [nch, n] uint8 CUDA -> [nch, ceil(n / 8)] MSB-first bytes."""
        bits = bits.contiguous()
        nch, n = bits.shape
        nb = (n + 7) // 8
        out = torch.empty((nch, max(nb, 1)), dtype=torch.uint8, device=bits.device)
        torch.cuda.current_stream().synchronize()
        _lib.check(self.h, self.L.dsdgpu_pack_native(self.h, nch, C.c_void_p(bits.data_ptr()),
                                                     bits.stride(0), n, C.c_void_p(out.data_ptr()),
                                                     out.stride(0)))
        return out[:, :nb]
