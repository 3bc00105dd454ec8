"""Batched multi-stream conversion over libdsdgpu's plan API.

`BatchPlan` converts many whole PCM streams (uneven lengths, mixed rates,
mixed NTFs) in one pass: per-stream FIR chains, one persistent SDM launch per
trellis parameter set over every DAS segment of every stream, one seam-search
launch, per-stream assembly and packing, replayed from CUDA graphs.  Streams
marked `precorr` run the PreCorr greedy SDM instead (one launch per PreCorr
parameter set over all such channels, one thread each).  Each
stream's output equals the single-stream pipeline (dsdgpu_pipeline_process,
the reference's plugin PCM path src/dsp_plugin.c:2990-3216 with full-parallel
DAS) run on a fresh context with the same parameters.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .ntf import NtfFilter

OUT_BITS, OUT_DOP, OUT_NATIVE = _lib.OUT_BITS, _lib.OUT_DOP, _lib.OUT_NATIVE


@dataclass
class StreamSpec:
    fs_in: int
    fs_out: int
    channels: int
    frames: int
    ntf: NtfFilter
    cands: int = 32
    depth: int = 64
    lat: int = 128
    state_limit: float = 0.0
    gain: float = 1.0
    boxcar_taps: int = 8
    soft_clip: bool = True
    reposition: bool = True
    precorr: bool = False      # PreCorr greedy SDM instead of the DAS trellis
    lowpass: bool = False      # same-rate DSD input: the 127-tap FIR lowpass, not the boxcar

    def desc(self) -> _lib.StreamDesc:
        d = _lib.StreamDesc()
        d.fs_in, d.fs_out, d.channels = self.fs_in, self.fs_out, self.channels
        d.boxcar_taps, d.frames, d.gain = self.boxcar_taps, self.frames, float(self.gain)
        d.soft_clip, d.reposition = int(self.soft_clip), int(self.reposition)
        d.sdm.order = self.ntf.order
        for i in range(self.ntf.order):
            d.sdm.a[i] = float(self.ntf.a[i])
            d.sdm.g[i] = float(self.ntf.g[i])
        d.sdm.depth, d.sdm.cands, d.sdm.lat = self.depth, self.cands, self.lat
        d.sdm.state_limit = float(self.state_limit)
        d.sdm_mode = _lib.SDM_PRECORR if self.precorr else _lib.SDM_TRELLIS
        d.samerate_filter = _lib.SAMERATE_LOWPASS if self.lowpass else _lib.SAMERATE_BOXCAR
        return d


class _Cai:
    """A device buffer described by __cuda_array_interface__ (for torch.as_tensor)."""

    def __init__(self, ptr: int, shape, typestr: str, strides=None):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 3,
                                         "strides": None if strides is None else tuple(strides)}


class BatchPlan:
    def __init__(self, specs: list[StreamSpec], seg_len: int = 0, output_format: int = OUT_DOP,
                 device: int = 0, max_device_bytes: int = 0, select: int | None = None,
                 lanes: int | None = None):
        self.L = _lib.load()
        self.device = device
        self.specs = list(specs)
        self.fmt = output_format
        h = C.c_void_p()
        rc = self.L.dsdgpu_create(device, C.byref(h))
        if rc != _lib.OK:
            raise _lib.DsdGpuError(rc, "dsdgpu_create failed")
        self.h = h
        self.plan = None
        if select is not None:
            _lib.check(self.h, self.L.dsdgpu_set_option(self.h, _lib.OPT_SDM_SELECT, select))
        if lanes is not None:   # lanes of a warp per trellis job (a power of two >= K)
            _lib.check(self.h, self.L.dsdgpu_set_option(self.h, _lib.OPT_SDM_LANES, lanes))
        arr = (_lib.StreamDesc * len(specs))(*[s.desc() for s in specs])
        p = C.c_void_p()
        _lib.check(self.h, self.L.dsdgpu_plan_create(self.h, arr, len(specs), seg_len,
                                                     output_format, max_device_bytes, C.byref(p)))
        self.plan = p
        self._streams = [self._stream(i) for i in range(len(specs))]

    def _stream(self, i: int) -> dict:
        pcm, pstride, out = C.c_void_p(), C.c_size_t(), C.c_void_p()
        ostride, nsmp, nbytes = C.c_size_t(), C.c_size_t(), C.c_size_t()
        _lib.check(self.h, self.L.dsdgpu_plan_stream(self.plan, i, C.byref(pcm), C.byref(pstride),
                                                     C.byref(out), C.byref(ostride),
                                                     C.byref(nsmp), C.byref(nbytes)))
        return {"pcm": pcm.value, "pcm_stride": pstride.value, "out": out.value,
                "out_stride": ostride.value, "out_samples": nsmp.value, "out_bytes": nbytes.value}

    # -- plan facts --
    def info(self) -> dict:
        pi = _lib.PlanInfo()
        _lib.check(self.h, self.L.dsdgpu_plan_info(self.plan, C.byref(pi)))
        return {k: getattr(pi, k) for k, _ in _lib.PlanInfo._fields_}

    def out_samples(self, i: int) -> int:
        return self._streams[i]["out_samples"]

    def out_bytes(self, i: int) -> int:
        return self._streams[i]["out_bytes"]

    # -- device buffers --
    def pcm_view(self, i: int) -> torch.Tensor:
        """The plan's PCM input of stream i: float32 [channels, frames] on the device."""
        s, sp = self._streams[i], self.specs[i]
        cai = _Cai(s["pcm"], (sp.channels, sp.frames), "<f4", (s["pcm_stride"] * 4, 4))
        return torch.as_tensor(cai, device=f"cuda:{self.device}")

    def out_view(self, i: int) -> torch.Tensor:
        """Stream i's packed output on the device: DoP bytes [out_bytes], NATIVE
        [channels, out_stride] rows, BITS [channels, out_samples] decision bytes."""
        s, sp = self._streams[i], self.specs[i]
        dev = f"cuda:{self.device}"
        if self.fmt == OUT_DOP:
            return torch.as_tensor(_Cai(s["out"], (s["out_bytes"],), "|u1"), device=dev)
        if self.fmt == OUT_NATIVE:
            return torch.as_tensor(_Cai(s["out"], (sp.channels, s["out_stride"]), "|u1",
                                        (s["out_stride"], 1)), device=dev)
        return torch.as_tensor(_Cai(s["out"], (sp.channels, s["out_samples"]), "|u1",
                                    (s["out_stride"], 1)), device=dev)

    def load(self, pcms) -> None:
        """Copy each stream's float32 [channels, frames] CUDA tensor into the plan."""
        for i, x in enumerate(pcms):
            self.pcm_view(i).copy_(x)
        torch.cuda.current_stream(self.device).synchronize()

    # -- runs --
    def run(self) -> None:
        torch.cuda.current_stream(self.device).synchronize()
        _lib.check(self.h, self.L.dsdgpu_plan_run(self.plan))

    def run_host(self, pcms: list[np.ndarray], outs: list[np.ndarray] | None = None):
        """Host buffers in and out (copies inside the call); returns the outputs."""
        n = len(self.specs)
        ins = [np.ascontiguousarray(x, np.float32) for x in pcms]
        if outs is None:
            outs = [np.empty(self.out_bytes(i), np.uint8) for i in range(n)]
        pin = (C.c_void_p * n)(*[x.ctypes.data for x in ins])
        pout = (C.c_void_p * n)(*[o.ctypes.data for o in outs])
        _lib.check(self.h, self.L.dsdgpu_plan_run_host(self.plan, pin, pout))
        return outs

    def times_ms(self) -> dict:
        t = (C.c_float * 4)()
        _lib.check(self.h, self.L.dsdgpu_plan_times(self.plan, t))
        return {"fir_rms": t[0], "sdm": t[1], "stitch_pack": t[2], "total": t[3]}

    def time_plain(self, njobs: int) -> tuple[int, float]:
        smp, sec = C.c_int64(), C.c_double()
        _lib.check(self.h, self.L.dsdgpu_plan_time_plain(self.plan, njobs, C.byref(smp),
                                                         C.byref(sec)))
        return smp.value, sec.value

    def launches(self) -> int:
        v = C.c_uint64()
        _lib.check(self.h, self.L.dsdgpu_launch_count(self.h, C.byref(v)))
        return v.value

    def sdm_work(self) -> tuple[int, int]:
        a, b = C.c_uint64(), C.c_uint64()
        _lib.check(self.h, self.L.dsdgpu_sdm_work(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def close(self):
        if getattr(self, "plan", None):
            self.L.dsdgpu_plan_destroy(self.plan)
            self.plan = None
        if getattr(self, "h", None):
            self.L.dsdgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
