"""Host-side mirror of the reference's trellis SDM interface over libdsdgpu.

`TrellisSdm` holds a bank of device SDM contexts (one per channel or DAS
segment) and exposes the reference's per-context operations with the same
names and meanings (include/trellis.h:62-88): process_block, drain,
copy_state, reset, plus the batched `segments` call (sdm_segment_process over
many contexts in one persistent launch).  Device buffers are torch CUDA
tensors (plumbing only); every computation runs in libdsdgpu's kernels.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib


def _sync_torch():
    torch.cuda.current_stream().synchronize()


@dataclass
class SegmentSpec:
    """One dsdgpu_segment_t: sdm_segment_process(ctx, in, out, count, discard)."""
    x: torch.Tensor                 # float64 CUDA, the segment's input
    channel: int
    discard: int = 0
    seed_from: int = -1
    seed_state: torch.Tensor | None = None   # float64 CUDA, `order` values


class TrellisSdm:
    def __init__(self, order: int, a, g, depth: int, cands: int, lat: int,
                 state_limit: float = 0.0, num_contexts: int = 1, device: int = 0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.dsdgpu_create(device, C.byref(h))
        if rc != _lib.OK:
            raise _lib.DsdGpuError(rc, "dsdgpu_create failed")
        self.h = h
        self.device = device
        p = _lib.SdmParams()
        p.order = order
        for i in range(order):
            p.a[i] = float(a[i])
            p.g[i] = float(g[i])
        p.depth, p.cands, p.lat = depth, cands, lat
        p.state_limit = float(state_limit)
        _lib.check(self.h, self.L.dsdgpu_sdm_setup(self.h, C.byref(p), num_contexts))
        self.order, self.depth, self.cands, self.lat = order, depth, cands, lat
        self.num_contexts = num_contexts

    def set_select(self, mode: int) -> None:
        """Survivor selection: _lib.SELECT_FAST (default), SELECT_EXACT, SELECT_VERIFY."""
        _lib.check(self.h, self.L.dsdgpu_set_option(self.h, _lib.OPT_SDM_SELECT, mode))

    def set_option(self, option: int, value: int) -> None:
        _lib.check(self.h, self.L.dsdgpu_set_option(self.h, option, value))

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

    # -- sdm_process_block over channels [first, first + nch) --
    def process_block(self, x: torch.Tensor, first: int = 0) -> list[torch.Tensor]:
        """x: [nch, count] float64 on this device; returns per-channel uint8 decisions."""
        x = x.to(torch.float64).contiguous()
        if x.dim() == 1:
            x = x.unsqueeze(0)
        nch, count = x.shape
        out = torch.empty((nch, max(count, 1)), dtype=torch.uint8, device=x.device)
        oc = (C.c_size_t * nch)()
        _sync_torch()
        _lib.check(self.h, self.L.dsdgpu_sdm_process(
            self.h, first, nch, C.c_void_p(x.data_ptr()), count, count,
            C.c_void_p(out.data_ptr()), out.shape[1], oc))
        return [out[c, : oc[c]] for c in range(nch)]

    def process_block_host(self, x: np.ndarray, first: int = 0) -> list[np.ndarray]:
        """Host-buffer form: float64 [nch, count] in, float32 +-1.0 out."""
        x = np.ascontiguousarray(np.atleast_2d(x), np.float64)
        nch, count = x.shape
        out = np.zeros((nch, max(count, 1)), np.float32)
        oc = (C.c_size_t * nch)()
        _lib.check(self.h, self.L.dsdgpu_sdm_process_host(
            self.h, first, nch, x.ctypes.data_as(C.c_void_p), count,
            out.ctypes.data_as(C.c_void_p), oc))
        return [out[c, : oc[c]] for c in range(nch)]

    def drain(self, max_out: int, first: int = 0, nch: int = 1) -> list[torch.Tensor]:
        out = torch.empty((nch, max(max_out, 1)), dtype=torch.uint8,
                          device=f"cuda:{self.device}")
        oc = (C.c_size_t * nch)()
        _sync_torch()
        _lib.check(self.h, self.L.dsdgpu_sdm_drain(
            self.h, first, nch, C.c_void_p(out.data_ptr()), out.shape[1], max_out, oc))
        return [out[c, : oc[c]] for c in range(nch)]

    def copy_state(self, dst: int, src: int) -> None:
        _lib.check(self.h, self.L.dsdgpu_sdm_copy_state(self.h, dst, src))

    def reset(self, channel: int = -1) -> None:
        _lib.check(self.h, self.L.dsdgpu_sdm_reset(self.h, channel))

    def segments(self, specs: list[SegmentSpec]) -> list[torch.Tensor]:
        """sdm_segment_process on every spec in one persistent launch."""
        n = len(specs)
        arr = (_lib.Segment * n)()
        outs = []
        for i, s in enumerate(specs):
            x = s.x
            assert x.dtype == torch.float64 and x.is_cuda and x.is_contiguous()
            o = torch.empty(max(x.numel(), 1), dtype=torch.uint8, device=x.device)
            outs.append(o)
            arr[i].d_in = x.data_ptr()
            arr[i].d_out = o.data_ptr()
            arr[i].count = x.numel()
            arr[i].discard = s.discard
            arr[i].channel = s.channel
            arr[i].seed_from = s.seed_from
            arr[i].d_seed_state = s.seed_state.data_ptr() if s.seed_state is not None else None
        _sync_torch()
        _lib.check(self.h, self.L.dsdgpu_sdm_segments(self.h, arr, n))
        return [outs[i][: arr[i].out_count] for i in range(n)]

    def query(self, channel: int) -> dict:
        st = (C.c_double * 10)()
        info = (C.c_uint64 * 6)()
        _lib.check(self.h, self.L.dsdgpu_sdm_query(self.h, channel, st, info))
        return {"best_state": np.array(st[: self.order]), "conv_fail": info[0],
                "cands_collapse": info[1], "next_filter_drops": info[2],
                "total_children": info[3], "num_cands": info[4], "pending": info[5]}
