"""Differentiable PCM -> DSD path over libdsdgpu's dsdgpu_diff_* entry points.

`DiffEngine` runs the forward (pre-emphasis FIR -> FP64 upsampling chain ->
exact trellis SDM -> in-band loss) and the hand-written straight-through
adjoint on the GPU.  `SdmLoss` wraps it as a torch.autograd.Function so a
training loop can optimise the pre-emphasis taps and the NTF coefficients the
way the reference's training_pipeline does with its soft SDM
(training_pipeline/diff_sdm.py:42-168), but against the exact trellis
decisions: the forward bits stay exact, the quantiser is relaxed only in the
gradient (y = y^ + kappa (v - v^)).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .ntf import NtfFilter


@dataclass
class DiffConfig:
    fs_in: int = 44100
    fs_out: int = 5644800
    nclips: int = 16
    frames: int = 8192
    preemph_taps: int = 127
    decim: int = 64
    lpf_taps: int = 255
    lpf_cutoff_hz: float = 20000.0
    kappa: float = 1.0
    gain: float = 0.5
    checkpoint: int = 4096
    cands: int = 32
    depth: int = 64
    lat: int = 128

    def abi(self, f: NtfFilter) -> _lib.DiffParams:
        p = _lib.DiffParams()
        p.fs_in, p.fs_out, p.nclips = self.fs_in, self.fs_out, self.nclips
        p.preemph_taps, p.frames, p.decim = self.preemph_taps, self.frames, self.decim
        p.lpf_taps, p.lpf_cutoff_hz, p.kappa = self.lpf_taps, self.lpf_cutoff_hz, self.kappa
        p.gain, p.checkpoint = self.gain, self.checkpoint
        p.sdm.order = f.order
        for i in range(f.order):
            p.sdm.a[i] = float(f.a[i])
            p.sdm.g[i] = float(f.g[i])
        p.sdm.depth, p.sdm.cands, p.sdm.lat = self.depth, self.cands, self.lat
        return p


def _arr(x, n=None) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(x, np.float64).reshape(-1))
    if n is not None:
        assert a.size == n
    return a


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class DiffEngine:
    def __init__(self, cfg: DiffConfig, ntf: NtfFilter, device: int = 0):
        self.L = _lib.load()
        self.cfg, self.ntf, self.order, self.device = cfg, ntf, ntf.order, device
        h = C.c_void_p()
        rc = self.L.dsdgpu_create(device, C.byref(h))
        if rc != _lib.OK:
            raise _lib.DsdGpuError(rc, "dsdgpu_create failed")
        self.h = h
        self.d = None
        p = cfg.abi(ntf)
        d = C.c_void_p()
        _lib.check(self.h, self.L.dsdgpu_diff_create(self.h, C.byref(p), C.byref(d)))
        self.d = d

    def set_input(self, pcm: torch.Tensor) -> None:
        """pcm: float32 [nclips, frames] on this device."""
        x = pcm.to(torch.float32).contiguous()
        assert tuple(x.shape) == (self.cfg.nclips, self.cfg.frames)
        torch.cuda.current_stream(self.device).synchronize()
        _lib.check(self.h, self.L.dsdgpu_diff_set_input(self.d, C.c_void_p(x.data_ptr())))

    def forward(self, taps, a, g) -> float:
        t, aa, gg = _arr(taps, self.cfg.preemph_taps), _arr(a, self.order), _arr(g, self.order)
        out = C.c_double()
        _lib.check(self.h, self.L.dsdgpu_diff_forward(self.d, _dp(t), _dp(aa), _dp(gg), C.byref(out)))
        return out.value

    def backward(self):
        gt = np.zeros(self.cfg.preemph_taps)
        ga, gg = np.zeros(self.order), np.zeros(self.order)
        _lib.check(self.h, self.L.dsdgpu_diff_backward(self.d, _dp(gt), _dp(ga), _dp(gg)))
        return gt, ga, gg

    def surrogate(self, taps, a, g) -> float:
        t, aa, gg = _arr(taps, self.cfg.preemph_taps), _arr(a, self.order), _arr(g, self.order)
        out = C.c_double()
        _lib.check(self.h, self.L.dsdgpu_diff_surrogate(self.d, _dp(t), _dp(aa), _dp(gg), C.byref(out)))
        return out.value

    def times_ms(self) -> dict:
        t = (C.c_float * 4)()
        _lib.check(self.h, self.L.dsdgpu_diff_times(self.d, t))
        return {"forward": t[0], "exact_sdm": t[1], "adjoint": t[2], "surrogate": t[3]}

    def buffers(self):
        """(SDM input float64 [nclips, n], decisions uint8 [nclips, n]) of the last forward, copied."""
        u, b, n = C.c_void_p(), C.c_void_p(), C.c_int64()
        _lib.check(self.h, self.L.dsdgpu_diff_buffers(self.d, C.byref(u), C.byref(b), C.byref(n)))
        from .batch import _Cai
        nc, nn = self.cfg.nclips, n.value
        dev = f"cuda:{self.device}"
        uu = torch.as_tensor(_Cai(u.value, (nc, nn), "<f8"), device=dev).clone()
        bb = torch.as_tensor(_Cai(b.value, (nc, nn), "|u1"), device=dev).clone()
        return uu, bb

    def launches(self) -> int:
        v = C.c_uint64()
        _lib.check(self.h, self.L.dsdgpu_launch_count(self.h, C.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "d", None):
            self.L.dsdgpu_diff_destroy(self.d)
            self.d = None
        if getattr(self, "h", None):
            self.L.dsdgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _SdmLossFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, taps, a, g, engine):
        loss = engine.forward(taps.detach().double().cpu().numpy(), a.detach().double().cpu().numpy(),
                              g.detach().double().cpu().numpy())
        ctx.engine = engine
        ctx.meta = (taps.dtype, taps.device, a.dtype, a.device, g.dtype, g.device)
        return torch.tensor(loss, dtype=torch.float64, device=a.device)

    @staticmethod
    def backward(ctx, gout):
        gt, ga, gg = ctx.engine.backward()
        td, tdev, ad, adev, gd, gdev = ctx.meta
        s = float(gout)
        return (torch.from_numpy(gt * s).to(dtype=td, device=tdev),
                torch.from_numpy(ga * s).to(dtype=ad, device=adev),
                torch.from_numpy(gg * s).to(dtype=gd, device=gdev), None)


class SdmLoss(torch.nn.Module):
    """In-band loss of the exact trellis SDM output with trainable pre-emphasis
    taps (float32, initialised to a unit impulse plus N(0, init_std)) and NTF
    coefficients a, g (float64)."""

    def __init__(self, cfg: DiffConfig, ntf: NtfFilter, device: int = 0, init_std: float = 1e-3,
                 seed: int = 0):
        super().__init__()
        self.engine = DiffEngine(cfg, ntf, device)
        gen = torch.Generator().manual_seed(seed)
        w = torch.randn(cfg.preemph_taps, generator=gen, dtype=torch.float64) * init_std
        w[0] += 1.0
        self.taps = torch.nn.Parameter(w.float())
        self.a = torch.nn.Parameter(torch.tensor(ntf.a[: ntf.order], dtype=torch.float64))
        self.g = torch.nn.Parameter(torch.tensor(ntf.g[: ntf.order], dtype=torch.float64))

    def set_input(self, pcm: torch.Tensor) -> None:
        self.engine.set_input(pcm)

    def forward(self) -> torch.Tensor:
        return _SdmLossFn.apply(self.taps, self.a, self.g, self.engine)
