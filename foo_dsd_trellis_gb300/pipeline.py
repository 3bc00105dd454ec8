"""Host-side mirror of the reference's PCM/DSD -> DSD conversion with DAS.

`Encoder` drives libdsdgpu's whole-path entry points: FIR chain with the
engine glue (boxcar, gain ramp, soft clip), segment-parallel trellis SDM with
Density-Aligned Stitching (or PreCorr), and DoP / native packing — the GPU
counterpart of plugin_process_pcm with the DAS phases of plugin_process
(reference src/dsp_plugin.c:2990-3216, 1283-2945) and of engine_process_block's
DSD branches (src/engine.c:479-729).

The input follows the rates, as the engine decides: below 2,822,400 Hz it is
planar float32 PCM; at or above it, planar DoP floats (16 DSD samples a frame),
re-encoded at the same rate (boxcar or, with samerate_filter, the FIR
lowpass), converted to a higher DSD rate (FIR upsampling on the +-1 input) or
a lower one (FP64 decimation), or decimated to PCM with output_format OUT_PCM.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib, ntf

OUT_BITS, OUT_DOP, OUT_NATIVE = _lib.OUT_BITS, _lib.OUT_DOP, _lib.OUT_NATIVE
FULL_PARALLEL, SEG0_FIRST = _lib.DAS_FULL_PARALLEL, _lib.DAS_SEG0_FIRST

# engine_channel_init: PCM rate conversion has no path-table entry, so the
# FIR gain is the -3 dB default halved (src/engine.c:206-210, dsd_types.h:450-460)
PCM_FIR_GAIN = float(np.float32(np.float32(0.708) * np.float32(0.5)))


class Encoder:
    def __init__(self, fs_in: int, fs_out: int, num_channels: int, ntf_filter: ntf.NtfFilter,
                 depth: int, cands: int, lat: int, state_limit: float = 0.0,
                 seg_len: int = 65536, nsegs: int = 0, seed_mode: int = FULL_PARALLEL,
                 reposition: bool = True, boxcar_taps: int = 8, soft_clip: bool = True,
                 output_format: int = OUT_DOP, sdm_mode: int = _lib.SDM_TRELLIS,
                 samerate_filter: int = _lib.SAMERATE_BOXCAR, device: int = 0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.dsdgpu_create(device, C.byref(h))
        if rc != _lib.OK:
            raise _lib.DsdGpuError(rc, "dsdgpu_create failed")
        self.h = h
        p = _lib.PipelineParams()
        p.fir.fs_in, p.fir.fs_out = fs_in, fs_out
        p.fir.boxcar_taps, p.fir.soft_clip = boxcar_taps, int(soft_clip)
        f = ntf_filter
        p.sdm.order = f.order
        for i in range(f.order):
            p.sdm.a[i] = f.a[i]
            p.sdm.g[i] = f.g[i]
        p.sdm.depth, p.sdm.cands, p.sdm.lat = depth, cands, lat
        p.sdm.state_limit = float(state_limit)
        p.das.seg_len, p.das.nsegs = seg_len, nsegs
        p.das.seed_mode, p.das.reposition = seed_mode, int(reposition)
        p.output_format = output_format
        p.sdm_mode = sdm_mode
        p.samerate_filter = samerate_filter
        _lib.check(self.h, self.L.dsdgpu_pipeline_setup(self.h, C.byref(p), num_channels))
        self.params = p
        self.nch = num_channels
        # DSD input (fs_in at or above DSD64) is DoP, 16 DSD samples per frame
        dsd_in = fs_in >= 2822400
        if output_format == _lib.OUT_PCM:
            self.ratio = 16 / (fs_in // fs_out)
        elif dsd_in:
            self.ratio = 16 * fs_out / fs_in
        else:
            self.ratio = fs_out // fs_in
        self.output_format = output_format
        self.device = device
        s = C.c_void_p()
        _lib.check(self.h, self.L.dsdgpu_get_stream(self.h, C.byref(s)))
        self.stream_ptr = s.value

    def close(self):
        if getattr(self, "h", None):
            self.L.dsdgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def out_capacity(self, frames: int) -> int:
        n = int(frames * self.ratio)
        if self.output_format == _lib.OUT_PCM:
            return 4 * n * self.nch
        if self.output_format == OUT_DOP:
            return (n // 16) * 3 * self.nch
        if self.output_format == OUT_NATIVE:
            return ((n + 7) // 8) * self.nch
        return n * self.nch

    def set_conv(self, ir, partition: int = 4096) -> None:
        """Convolve every channel with its IR (float32 [nch, taps]) between the
        FIR chain and the SDM (UPOLS, FP32)."""
        from . import conv
        conv.setup(self.L, self.h, ir, partition)

    def flush(self) -> None:
        """Start a new stream (plugin_flush, src/dsp_plugin.c:3622-3653): SDM
        state, filter histories and the DoP marker phase are reset."""
        _lib.check(self.h, self.L.dsdgpu_pipeline_flush(self.h))

    def process(self, pcm: torch.Tensor, out: torch.Tensor, gain_start: float = PCM_FIR_GAIN,
                gain_end: float = PCM_FIR_GAIN):
        """Device buffers: pcm [nch, frames] float32; out a uint8 tensor whose rows
        are out.stride(0) bytes (any layout for DoP).  Returns (samples, bytes)."""
        nch, frames = pcm.shape
        ns, nb = C.c_size_t(), C.c_size_t()
        stride = out.stride(0) if out.dim() > 1 else out.numel()
        _lib.check(self.h, self.L.dsdgpu_pipeline_process(
            self.h, C.c_void_p(pcm.data_ptr()), pcm.stride(0), frames, gain_start, gain_end,
            C.c_void_p(out.data_ptr()), stride, C.byref(ns), C.byref(nb)))
        return ns.value, nb.value

    def process_host(self, pcm: np.ndarray, out: np.ndarray, gain_start: float = PCM_FIR_GAIN,
                     gain_end: float = PCM_FIR_GAIN):
        """Host buffers (planar float32 PCM in, packed bytes out), copies included."""
        ns, nb = C.c_size_t(), C.c_size_t()
        _lib.check(self.h, self.L.dsdgpu_pipeline_process_host(
            self.h, C.c_void_p(pcm.ctypes.data), pcm.shape[1], gain_start, gain_end,
            C.c_void_p(out.ctypes.data), out.nbytes, C.byref(ns), C.byref(nb)))
        return ns.value, nb.value

    def launches(self) -> int:
        v = C.c_uint64()
        _lib.check(self.h, self.L.dsdgpu_launch_count(self.h, C.byref(v)))
        return v.value

    def last_sdm_kernel(self) -> str:
        return _lib.last_sdm_kernel(self.h)

    def sdm_work(self):
        t, l = C.c_uint64(), C.c_uint64()
        _lib.check(self.h, self.L.dsdgpu_sdm_work(self.h, C.byref(t), C.byref(l)))
        return t.value, l.value

    def probe_fp64_gops(self) -> float:
        v = C.c_double()
        _lib.check(self.h, self.L.dsdgpu_probe_fp64(self.h, C.byref(v)))
        return v.value

    def stage_ms(self) -> dict:
        v = (C.c_float * 5)()
        _lib.check(self.h, self.L.dsdgpu_stage_times(self.h, v))
        return {"fir": v[0], "sdm": v[1], "das": v[2], "pack": v[3], "total": v[4]}
