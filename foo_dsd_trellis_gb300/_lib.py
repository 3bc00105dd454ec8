"""ctypes binding of libdsdgpu.so (include/dsdgpu.h).

The library is built in-tree by foo_dsd_trellis_gb300/build.py.  Loading fails
loudly when it is missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libdsdgpu.so")

OK = 0
ERR_ARG = -1
ERR_CUDA = -2
ERR_NOMEM = -3
ERR_STATE = -4
ERR_DEVICE = -5
ERR_UNSUPPORTED = -6
ERR_TOO_LARGE = -7

_ERR_NAMES = {ERR_ARG: "ERR_ARG", ERR_CUDA: "ERR_CUDA", ERR_NOMEM: "ERR_NOMEM",
              ERR_STATE: "ERR_STATE", ERR_DEVICE: "ERR_DEVICE",
              ERR_UNSUPPORTED: "ERR_UNSUPPORTED", ERR_TOO_LARGE: "ERR_TOO_LARGE"}


class DsdGpuError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{_ERR_NAMES.get(code, code)}: {message}")
        self.code = code


class SdmParams(C.Structure):
    _fields_ = [("order", C.c_int), ("a", C.c_double * 10), ("g", C.c_double * 10),
                ("depth", C.c_int), ("cands", C.c_int), ("lat", C.c_int),
                ("state_limit", C.c_double)]


class Segment(C.Structure):
    _fields_ = [("d_in", C.c_void_p), ("d_out", C.c_void_p), ("count", C.c_int64),
                ("discard", C.c_int64), ("channel", C.c_int), ("seed_from", C.c_int),
                ("d_seed_state", C.c_void_p), ("out_count", C.c_int64)]


class EstimateItem(C.Structure):
    _fields_ = [("d_in", C.c_void_p), ("count", C.c_int64), ("init_state", C.c_double * 10),
                ("out_state", C.c_double * 10)]


class FirParams(C.Structure):
    _fields_ = [("fs_in", C.c_uint), ("fs_out", C.c_uint), ("boxcar_taps", C.c_int),
                ("soft_clip", C.c_int)]


class DasParams(C.Structure):
    _fields_ = [("seg_len", C.c_int64), ("nsegs", C.c_int), ("seed_mode", C.c_int),
                ("reposition", C.c_int)]


class PipelineParams(C.Structure):
    _fields_ = [("fir", FirParams), ("sdm", SdmParams), ("das", DasParams),
                ("output_format", C.c_int), ("sdm_mode", C.c_int), ("samerate_filter", C.c_int)]


class StreamDesc(C.Structure):
    _fields_ = [("fs_in", C.c_int32), ("fs_out", C.c_int32), ("channels", C.c_int32),
                ("boxcar_taps", C.c_int32), ("frames", C.c_int64), ("gain", C.c_double),
                ("soft_clip", C.c_int32), ("reposition", C.c_int32), ("sdm", SdmParams),
                ("sdm_mode", C.c_int32), ("samerate_filter", C.c_int32)]


class PlanInfo(C.Structure):
    _fields_ = [("seg_len", C.c_int64), ("jobs", C.c_int64), ("sdm_samples", C.c_int64),
                ("out_samples", C.c_int64), ("device_bytes", C.c_int64),
                ("classes", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("predicted_ms", C.c_double)]


class DiffParams(C.Structure):
    _fields_ = [("fs_in", C.c_int32), ("fs_out", C.c_int32), ("nclips", C.c_int32),
                ("preemph_taps", C.c_int32), ("frames", C.c_int64), ("decim", C.c_int32),
                ("lpf_taps", C.c_int32), ("lpf_cutoff_hz", C.c_double), ("kappa", C.c_double),
                ("gain", C.c_double), ("checkpoint", C.c_int32), ("pad", C.c_int32),
                ("sdm", SdmParams)]


OUT_BITS = 0
OUT_DOP = 1
OUT_NATIVE = 2
OUT_PCM = 3
SDM_TRELLIS = 0
FILE_DSF = 1
FILE_DFF = 2
SDM_PRECORR = 1
SAMERATE_BOXCAR = 0
SAMERATE_LOWPASS = 1

OPT_SDM_SELECT = 1
OPT_SDM_LANES = 2
OPT_SDM_BALANCE = 3
OPT_FAILURE_TEST = 4
FAIL_PART_WAIT, FAIL_CHAIN_WALK = 1, 2
SELECT_FAST, SELECT_EXACT, SELECT_VERIFY = 0, 1, 2

DAS_FULL_PARALLEL = 0
DAS_SEG0_FIRST = 1


_vp = C.c_void_p
_sz = C.c_size_t
_szp = C.POINTER(C.c_size_t)
_dp = C.POINTER(C.c_double)

# name -> (restype, argtypes); the exported surface of include/dsdgpu.h
SIGNATURES = {
    "dsdgpu_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "dsdgpu_destroy": (None, [_vp]),
    "dsdgpu_last_error": (C.c_char_p, [_vp]),
    "dsdgpu_synchronize": (C.c_int, [_vp]),
    "dsdgpu_launch_count": (C.c_int, [_vp, C.POINTER(C.c_uint64)]),
    "dsdgpu_set_option": (C.c_int, [_vp, C.c_int, C.c_int]),
    "dsdgpu_sdm_work": (C.c_int, [_vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "dsdgpu_sdm_setup": (C.c_int, [_vp, C.POINTER(SdmParams), C.c_int]),
    "dsdgpu_sdm_reset": (C.c_int, [_vp, C.c_int]),
    "dsdgpu_sdm_process": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _sz, _sz, _vp, _sz, _szp]),
    "dsdgpu_sdm_process_host": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _sz, _vp, _szp]),
    "dsdgpu_sdm_drain": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _sz, _sz, _szp]),
    "dsdgpu_sdm_copy_state": (C.c_int, [_vp, C.c_int, C.c_int]),
    "dsdgpu_sdm_segments": (C.c_int, [_vp, C.POINTER(Segment), C.c_int]),
    "dsdgpu_sdm_last_kernel": (C.c_int, [_vp, C.c_char_p, _sz]),
    "dsdgpu_sdm_state_distance": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(C.c_double)]),
    "dsdgpu_sdm_estimate_state": (C.c_int, [_vp, C.POINTER(SdmParams), C.c_int,
                                            C.POINTER(EstimateItem), C.c_int]),
    "dsdgpu_sdm_query": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_double),
                                   C.POINTER(C.c_uint64)]),
    "dsdgpu_das_process": (C.c_int, [_vp, C.POINTER(DasParams), C.c_int, _vp, _sz, _sz, _vp,
                                     _sz, _szp, C.POINTER(C.c_int), C.c_int]),
    "dsdgpu_pack_dop": (C.c_int, [_vp, C.c_int, _vp, _sz, _sz, _vp, C.c_int,
                                  C.POINTER(C.c_int)]),
    "dsdgpu_pack_native": (C.c_int, [_vp, C.c_int, _vp, _sz, _sz, _vp, _sz]),
    "dsdgpu_pipeline_setup": (C.c_int, [_vp, C.POINTER(PipelineParams), C.c_int]),
    "dsdgpu_pipeline_flush": (C.c_int, [_vp]),
    "dsdgpu_pipeline_process": (C.c_int, [_vp, _vp, _sz, _sz, C.c_double, C.c_double, _vp, _sz,
                                          _szp, _szp]),
    "dsdgpu_pipeline_process_host": (C.c_int, [_vp, _vp, _sz, C.c_double, C.c_double, _vp, _sz,
                                               _szp, _szp]),
    "dsdgpu_stage_times": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "dsdgpu_get_stream": (C.c_int, [_vp, C.POINTER(_vp)]),
    "dsdgpu_sdm_process_noalloc": (C.c_int, [C.POINTER(SdmParams), C.c_int, C.c_int, _vp, _sz,
                                             _sz, _vp, _sz, _szp, _vp]),
    "dsdgpu_probe_fp64": (C.c_int, [_vp, C.POINTER(C.c_double)]),
    "dsdgpu_selftest_convert": (C.c_int, [_vp, C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64)]),
    "dsdgpu_plan_create": (C.c_int, [_vp, C.POINTER(StreamDesc), C.c_int, C.c_int64, C.c_int,
                                     C.c_uint64, C.POINTER(_vp)]),
    "dsdgpu_plan_destroy": (None, [_vp]),
    "dsdgpu_plan_info": (C.c_int, [_vp, C.POINTER(PlanInfo)]),
    "dsdgpu_plan_stream": (C.c_int, [_vp, C.c_int, C.POINTER(_vp), _szp, C.POINTER(_vp), _szp,
                                     _szp, _szp]),
    "dsdgpu_plan_run": (C.c_int, [_vp]),
    "dsdgpu_plan_run_host": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp)]),
    "dsdgpu_plan_times": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "dsdgpu_plan_time_plain": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int64),
                                         C.POINTER(C.c_double)]),
    "dsdgpu_dop_unpack": (C.c_int, [_vp, C.c_int, _vp, _sz, _sz, _vp, _sz]),
    "dsdgpu_dop_unpack_f32": (C.c_int, [_vp, C.c_int, _vp, _sz, _sz, _vp, _sz]),
    "dsdgpu_boxcar_setup": (C.c_int, [_vp, C.c_int, C.c_int]),
    "dsdgpu_boxcar_reset": (C.c_int, [_vp]),
    "dsdgpu_boxcar_process": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _sz, _sz, _vp, _sz,
                                        C.c_double, C.c_double]),
    "dsdgpu_boxcar_process_async": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _sz, _sz, _vp, _sz,
                                              C.c_double, C.c_double]),
    "dsdgpu_lowpass_setup": (C.c_int, [_vp, C.c_uint, C.c_double, C.c_int, C.c_int]),
    "dsdgpu_lowpass_taps": (C.c_int, [_vp, _vp, C.c_int, C.POINTER(C.c_int)]),
    "dsdgpu_lowpass_design": (C.c_int, [C.c_uint, C.c_double, C.c_int, _vp, C.c_int,
                                        C.POINTER(C.c_int)]),
    "dsdgpu_lowpass_reset": (C.c_int, [_vp]),
    "dsdgpu_lowpass_process": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _sz, _sz, _vp, _sz,
                                         C.c_double, C.c_double]),
    "dsdgpu_lowpass_process_async": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _sz, _sz, _vp, _sz,
                                               C.c_double, C.c_double]),
    "dsdgpu_decim_setup": (C.c_int, [_vp, C.c_uint, C.c_uint, C.c_int]),
    "dsdgpu_decim_reset": (C.c_int, [_vp]),
    "dsdgpu_decim_process_f64": (C.c_int, [_vp, C.c_int, _vp, _sz, _sz, _vp, _sz, C.c_double,
                                           C.c_double, C.c_int, C.POINTER(_sz)]),
    "dsdgpu_decim_process_f64_async": (C.c_int, [_vp, C.c_int, _vp, _sz, _sz, _vp, _sz,
                                                 C.c_double, C.c_double, C.c_int, C.POINTER(_sz)]),
    "dsdgpu_decim_process": (C.c_int, [_vp, C.c_int, _vp, _sz, _sz, _vp, _sz, C.c_double,
                                       C.c_double, _szp]),
    "dsdgpu_decim_process_async": (C.c_int, [_vp, C.c_int, _vp, _sz, _sz, _vp, _sz, C.c_double,
                                             C.c_double, _szp]),
    "dsdgpu_file_header": (C.c_int, [C.c_int, C.c_int, C.c_uint, C.c_uint64, _vp, _sz, _szp,
                                     C.POINTER(C.c_uint64)]),
    "dsdgpu_pack_file": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _sz, _sz, _vp,
                                   C.POINTER(C.c_uint64)]),
    "dsdgpu_precorr_setup": (C.c_int, [_vp, C.c_int, _vp, _vp, C.c_double, C.c_int]),
    "dsdgpu_precorr_reset": (C.c_int, [_vp]),
    "dsdgpu_precorr_table": (C.c_int, [_vp, _vp]),
    "dsdgpu_precorr_process": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _sz, _sz, _vp, _sz]),
    "dsdgpu_precorr_process_async": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _sz, _sz, _vp, _sz]),
    "dsdgpu_conv_setup": (C.c_int, [_vp, _vp, _sz, C.c_int, C.c_int]),
    "dsdgpu_conv_reset": (C.c_int, [_vp]),
    "dsdgpu_conv_clear": (C.c_int, [_vp]),
    "dsdgpu_conv_process": (C.c_int, [_vp, C.c_int, _vp, _sz, _sz, _vp, _sz]),
    "dsdgpu_diff_create": (C.c_int, [_vp, C.POINTER(DiffParams), C.POINTER(_vp)]),
    "dsdgpu_diff_destroy": (None, [_vp]),
    "dsdgpu_diff_set_input": (C.c_int, [_vp, _vp]),
    "dsdgpu_diff_forward": (C.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "dsdgpu_diff_backward": (C.c_int, [_vp, _dp, _dp, _dp]),
    "dsdgpu_diff_surrogate": (C.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "dsdgpu_diff_times": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "dsdgpu_diff_buffers": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(C.c_int64)]),
    "dsdgpu_fir_setup": (C.c_int, [_vp, C.POINTER(FirParams), C.c_int]),
    "dsdgpu_fir_reset": (C.c_int, [_vp]),
    "dsdgpu_fir_process": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _sz, _sz, _vp, _sz,
                                     C.c_double, C.c_double, _szp]),
    "dsdgpu_fir_process_async": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _sz, _sz, _vp, _sz,
                                           C.c_double, C.c_double, _szp]),
}

_lib = None


def load() -> C.CDLL:
    """Load libdsdgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first "
                           "(there is no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_sdm_kernel(ctx) -> str:
    """The kernel (with template arguments) of the context's last trellis SDM launch."""
    buf = C.create_string_buffer(64)
    check(ctx, load().dsdgpu_sdm_last_kernel(ctx, buf, 64))
    return buf.value.decode()


def check(ctx, rc: int) -> None:
    if rc != OK:
        msg = load().dsdgpu_last_error(ctx) if ctx else b""
        raise DsdGpuError(rc, (msg or b"").decode(errors="replace"))
