"""ORACLE — test infrastructure only.

ctypes bindings for oracle/liboracle.so (the C restatement) and, where it was
built, oracle/_ref/libref.so / libref_wide.so (the reference's own trellis.c,
ntf.c and dop.c).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
legs import this module; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_u8p = C.POINTER(C.c_uint8)
_u64p = C.POINTER(C.c_uint64)


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and the reference libraries when `ref`)."""
    subprocess.check_call(["make", "-s", "-C", HERE] + (["ref"] if ref else []),
                          stdout=subprocess.DEVNULL)


def _ptr(a, t):
    return a.ctypes.data_as(t)


class _SdmLib:
    """Common wrapper: `prefix` is 'ora' (restatement) or 'ref' (reference)."""

    def __init__(self, path: str, prefix: str):
        self.lib = C.CDLL(path)
        self.p = prefix
        L, p = self.lib, prefix
        f = getattr(L, f"{p}_sdm_new")
        f.restype = C.c_void_p
        f.argtypes = [C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_double]
        for name, res, args in [
            ("sdm_free", None, [C.c_void_p]),
            ("sdm_process", C.c_size_t, [C.c_void_p, _dp, _fp, C.c_size_t]),
            ("sdm_drain", C.c_size_t, [C.c_void_p, _fp, C.c_size_t]),
            ("sdm_reset", None, [C.c_void_p]),
            ("sdm_copy", None, [C.c_void_p, C.c_void_p]),
            ("sdm_segment", C.c_size_t, [C.c_void_p, _dp, _fp, C.c_size_t, C.c_size_t]),
            ("sdm_seed", None, [C.c_void_p, _dp]),
            ("sdm_best_state", None, [C.c_void_p, _dp]),
            ("sdm_info", None, [C.c_void_p, _u64p]),
            ("estimate_state", None, [C.c_int, _dp, _dp, _dp, _dp, C.c_size_t,
                                      C.c_double, C.c_int, _dp]),
            ("dop_pack_i24", C.c_int, [_fp, _u8p, C.c_size_t, C.c_int]),
            ("bits_pack", None, [_fp, _u8p, C.c_size_t]),
            ("sdm_cand", C.c_int, [C.c_void_p, C.c_uint, _dp, _dp, _u64p, C.POINTER(C.c_uint)]),
        ]:
            fn = getattr(L, f"{p}_{name}")
            fn.restype = res
            fn.argtypes = args
        self.lib.__dict__  # keep reference alive

    def fn(self, name):
        return getattr(self.lib, f"{self.p}_{name}")


class Sdm:
    """One trellis SDM context (the reference's sdm_context_t)."""

    def __init__(self, lib: _SdmLib, order, a, g, depth, cands, lat, state_limit=0.0):
        self.L = lib
        self.order = order
        self.a = np.zeros(10, np.float64)
        self.g = np.zeros(10, np.float64)
        self.a[:order] = a[:order]
        self.g[:order] = g[:order]
        self.h = lib.fn("sdm_new")(order, _ptr(self.a, _dp), _ptr(self.g, _dp), depth,
                                  cands, lat, float(state_limit))
        if not self.h:
            raise ValueError("sdm init rejected the parameters")
        self.lat = lat

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.L.fn("sdm_free")(h)
            self.h = None

    def process(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float64)
        out = np.empty(max(len(x), 1), np.float32)
        n = self.L.fn("sdm_process")(self.h, _ptr(x, _dp), _ptr(out, _fp), len(x))
        return out[:n]

    def segment(self, x: np.ndarray, discard: int) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float64)
        out = np.empty(max(len(x), 1), np.float32)
        n = self.L.fn("sdm_segment")(self.h, _ptr(x, _dp), _ptr(out, _fp), len(x), discard)
        return out[:n]

    def drain(self, max_out: int) -> np.ndarray:
        out = np.empty(max(max_out, 1), np.float32)
        n = self.L.fn("sdm_drain")(self.h, _ptr(out, _fp), max_out)
        return out[:n]

    def reset(self):
        self.L.fn("sdm_reset")(self.h)

    def copy_from(self, other: "Sdm"):
        self.L.fn("sdm_copy")(self.h, other.h)

    def seed(self, state):
        s = np.zeros(10, np.float64)
        s[: self.order] = state[: self.order]
        self.L.fn("sdm_seed")(self.h, _ptr(s, _dp))

    def best_state(self) -> np.ndarray:
        s = np.zeros(10, np.float64)
        self.L.fn("sdm_best_state")(self.h, _ptr(s, _dp))
        return s[: self.order]

    def cand(self, i: int):
        """Candidate i of the current bank: (state, cost, path, next)."""
        st = np.zeros(10, np.float64)
        cost = np.zeros(1, np.float64)
        path = np.zeros(1, np.uint64)
        nxt = C.c_uint()
        rc = self.L.fn("sdm_cand")(self.h, i, _ptr(st, _dp), _ptr(cost, _dp), _ptr(path, _u64p),
                                   C.byref(nxt))
        if rc != 0:
            raise IndexError(i)
        return st[: self.order], float(cost[0]), int(path[0]), int(nxt.value)

    def trace_row(self) -> bytes:
        """The current act list in order: cost (binary64), path, next of each
        candidate, packed little-endian."""
        import struct
        n = self.info()["num_cands"]
        return b"".join(struct.pack("<dQB", *self.cand(i)[1:]) for i in range(n))

    def info(self) -> dict:
        v = np.zeros(9, np.uint64)
        self.L.fn("sdm_info")(self.h, _ptr(v, _u64p))
        keys = ["num_cands", "pos", "pending", "idx", "draining", "conv_fail",
                "cands_collapse", "next_filter_drops", "total_children"]
        return {k: int(x) for k, x in zip(keys, v)}


_cache: dict = {}


def oracle_lib() -> _SdmLib:
    if "ora" not in _cache:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        lib = _SdmLib(path, "ora")
        _bind_oracle_extras(lib.lib)
        _cache["ora"] = lib
    return _cache["ora"]


def ref_lib(wide: bool = False):
    """The reference's own SDM, or None when oracle/_ref was not built."""
    key = "wide" if wide else "ref"
    if key not in _cache:
        path = os.path.join(REF_DIR, "libref_wide.so" if wide else "libref.so")
        if not os.path.exists(path):
            _cache[key] = None
        else:
            lib = _SdmLib(path, "ref")
            L = lib.lib
            L.ref_ntf_count.restype = C.c_int
            L.ref_ntf_entry.argtypes = [C.c_int, _dp, _dp, C.POINTER(C.c_int),
                                        C.POINTER(C.c_uint), C.c_char_p, C.c_int]
            L.ref_ntf_lookup.argtypes = [C.c_int, C.c_uint]
            L.ref_ntf_auto.argtypes = [C.c_uint]
            L.ref_path_bits.restype = C.c_int
            L.ref_dop_unpack.argtypes = [_fp, _fp, C.c_size_t]
            _cache[key] = lib
    return _cache[key]


class DasCfg(C.Structure):
    _fields_ = [("seg_len", C.c_int), ("nsegs", C.c_int), ("seed_mode", C.c_int),
                ("reposition", C.c_int)]


def das_run(order, a, g, depth, cands, lat, state_limit, fir: np.ndarray, seg_len=0, nsegs=0,
            seed_mode=0, reposition=True, nthreads=None, carry=None):
    """DAS over one chunk; fir is [nch, count] float64.  Returns (bits [nch, n],
    stitch positions per segment, segment starts).  carry: one Sdm per channel
    (the persistent contexts of a stream, fresh for its first chunk), updated
    in place for the next chunk."""
    L = oracle_lib().lib
    fir = np.ascontiguousarray(np.atleast_2d(fir), np.float64)
    nch, count = fir.shape
    aa = np.zeros(10); aa[:order] = a[:order]
    gg = np.zeros(10); gg[:order] = g[:order]
    cfg = DasCfg(seg_len, nsegs, seed_mode, int(reposition))
    outs = [np.zeros(count + 16, np.uint8) for _ in range(nch)]
    fps = (_dp * nch)(*[fir[c].ctypes.data_as(_dp) for c in range(nch)])
    ops = (_u8p * nch)(*[o.ctypes.data_as(_u8p) for o in outs])
    smax = max(1, (count // seg_len) if seg_len > 0 else nsegs)
    sp = (C.c_int * smax)()
    ss = (C.c_size_t * smax)()
    cp = None
    if carry is not None:
        if len(carry) != nch:
            raise ValueError("one carried context per channel")
        cp = (C.c_void_p * nch)(*[c.h for c in carry])
    n = L.ora_das_run_carry(order, _ptr(aa, _dp), _ptr(gg, _dp), depth, cands, lat,
                            float(state_limit), C.byref(cfg), fps, count, nch, ops, sp, ss,
                            nthreads or os.cpu_count() or 1, cp)
    return np.stack([o[:n] for o in outs]), list(sp), list(ss)


def dop_unpack(pcm: np.ndarray, lib=None) -> np.ndarray:
    """DoP float samples (one channel) -> +-1.0 float bits, 16 per sample."""
    pcm = np.ascontiguousarray(pcm, np.float32)
    out = np.empty(16 * len(pcm), np.float32)
    L = (lib or oracle_lib()).lib
    fn = L.ora_dop_unpack if lib is None else L.ref_dop_unpack
    fn(_ptr(pcm, _fp), _ptr(out, _fp), len(pcm))
    return out


class Boxcar:
    """The same-rate boxcar of the engine with its ring carried across calls."""

    def __init__(self, taps: int):
        self.L = oracle_lib().lib
        self.h = self.L.ora_boxcar_new(taps)

    def process(self, bits: np.ndarray, g_start: float, g_end: float) -> np.ndarray:
        bits = np.ascontiguousarray(bits, np.float32)
        out = np.empty(max(len(bits), 1), np.float64)
        self.L.ora_boxcar_gain(self.h, _ptr(bits, _fp), _ptr(out, _dp), len(bits),
                               float(g_start), float(g_end))
        return out[: len(bits)]

    def __del__(self):
        try:
            self.L.ora_boxcar_free(self.h)
        except Exception:
            pass


class Lowpass:
    """The same-rate FIR lowpass (fir_lowpass_init_ex + fir_lowpass_process,
    src/fir.c:795-872) with its delay line carried across calls and the
    engine's gain ramp."""

    def __init__(self, fs: int, cutoff_hz: float = 50000.0, ntaps: int = 127):
        self.L = oracle_lib().lib
        self.h = self.L.ora_lowpass_new(fs, float(cutoff_hz), ntaps)

    def taps(self) -> np.ndarray:
        h = np.zeros(256, np.float64)
        n = self.L.ora_lowpass_taps(self.h, _ptr(h, _dp))
        return h[:n]

    def process(self, bits: np.ndarray, g_start: float, g_end: float) -> np.ndarray:
        bits = np.ascontiguousarray(bits, np.float32)
        out = np.empty(max(len(bits), 1), np.float64)
        self.L.ora_lowpass_process(self.h, _ptr(bits, _fp), _ptr(out, _dp), len(bits),
                                   float(g_start), float(g_end))
        return out[: len(bits)]

    def __del__(self):
        try:
            self.L.ora_lowpass_free(self.h)
        except Exception:
            pass


def lowpass_design(fs: int, cutoff_hz: float = 50000.0, ntaps: int = 127) -> np.ndarray:
    h = np.zeros(256, np.float64)
    n = oracle_lib().lib.ora_lowpass_design(fs, float(cutoff_hz), ntaps, _ptr(h, _dp))
    return h[:n]


class PreCorr:
    """The PreCorr greedy SDM: the oracle's restatement, or (ref=True) the
    reference's own src/precorr.c compiled into oracle/_ref."""

    def __init__(self, order, a, g, state_limit=0.0, ref=False):
        aa = np.zeros(10); aa[:order] = a[:order]
        gg = np.zeros(10); gg[:order] = g[:order]
        self.ref = ref
        lib = ref_lib() if ref else oracle_lib()
        if lib is None:
            raise RuntimeError("reference build absent")
        self.L = lib.lib
        new = self.L.ref_precorr_new if ref else self.L.ora_precorr_new
        new.restype = C.c_void_p
        new.argtypes = [C.c_int, _dp, _dp, C.c_double]
        self.h = new(order, _ptr(aa, _dp), _ptr(gg, _dp), float(state_limit))

    def table(self) -> np.ndarray:
        t = np.zeros(256 * 8, np.float32)
        fn = self.L.ref_precorr_table if self.ref else self.L.ora_precorr_table
        fn.argtypes = [C.c_void_p, _fp]
        fn(self.h, _ptr(t, _fp))
        return t.reshape(256, 8)

    def process(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float64)
        if self.ref:
            f = np.zeros(max(len(x), 1), np.float32)
            self.L.ref_precorr_process.argtypes = [C.c_void_p, _dp, _fp, C.c_size_t]
            self.L.ref_precorr_process(self.h, _ptr(x, _dp), _ptr(f, _fp), len(x))
            return (f[: len(x)] > 0).astype(np.uint8)
        b = np.zeros(max(len(x), 1), np.uint8)
        self.L.ora_precorr_process.argtypes = [C.c_void_p, _dp, _u8p, C.c_size_t]
        self.L.ora_precorr_process(self.h, _ptr(x, _dp), _ptr(b, _u8p), len(x))
        return b[: len(x)]

    def __del__(self):
        try:
            (self.L.ref_precorr_free if self.ref else self.L.ora_precorr_free)(C.c_void_p(self.h))
        except Exception:
            pass


class Decimator:
    """The reference's DSD -> PCM FP64 decimation chain, streamed."""

    def __init__(self, fs_in: int, fs_out: int):
        self.L = oracle_lib().lib
        self.h = self.L.ora_decim_new(fs_in, fs_out)
        if not self.h:
            raise ValueError("unsupported rate pair")

    def process(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float64)
        out = np.empty(max(len(x), 1), np.float64)
        n = self.L.ora_decim_process(self.h, _ptr(x, _dp), len(x), _ptr(out, _dp))
        return out[:n]

    def __del__(self):
        try:
            self.L.ora_decim_free(self.h)
        except Exception:
            pass


def engine_down(bc: "Boxcar", dec: Decimator, x: np.ndarray, g_start: float, g_end: float,
                soft_clip: bool) -> np.ndarray:
    """DSD -> DSD downsampling branch of the engine: boxcar mean, FP64
    decimation, gain ramp, optional soft clip (state carried in bc and dec)."""
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty(max(len(x), 1), np.float64)
    n = oracle_lib().lib.ora_engine_down(bc.h, dec.h, _ptr(x, _fp), len(x), float(g_start),
                                         float(g_end), int(soft_clip), _ptr(out, _dp))
    return out[:n]


def dop_float_frames(bits01: np.ndarray, phase: int = 0) -> np.ndarray:
    """0/1 decision bytes -> DoP float samples (24-bit value / 2^23) with
    alternating markers, the format a decoder hands the plugin."""
    bits01 = np.asarray(bits01, np.uint8)
    frames = len(bits01) // 16
    w = np.zeros(frames, np.int64)
    for b in range(16):
        w = (w << 1) | bits01[b: 16 * frames: 16].astype(np.int64)
    marker = np.where((np.arange(frames) + phase) % 2 == 0, 0x05, 0xFA)
    v = (marker << 16) | w
    v = np.where(v >= 1 << 23, v - (1 << 24), v)
    return (v.astype(np.float64) / 8388608.0).astype(np.float32)


def _bind_oracle_extras(L):
    L.ora_sdm_process_bits.restype = C.c_size_t
    L.ora_sdm_process_bits.argtypes = [C.c_void_p, _dp, _u8p, C.c_size_t]
    L.ora_sdm_segment_bits.restype = C.c_size_t
    L.ora_sdm_segment_bits.argtypes = [C.c_void_p, _dp, _u8p, C.c_size_t, C.c_size_t]
    L.ora_dop_pack_u8.restype = C.c_int
    L.ora_dop_pack_u8.argtypes = [_u8p, _u8p, C.c_size_t, C.c_int]
    L.ora_bits_pack_u8.argtypes = [_u8p, _u8p, C.c_size_t]
    L.ora_fir_design.argtypes = [C.c_int, C.c_int, _dp]
    L.ora_fir_plan.argtypes = [C.c_uint, C.c_uint, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.ora_fir_upsample.restype = C.c_size_t
    L.ora_fir_upsample.argtypes = [C.c_uint, C.c_uint, _dp, C.c_size_t, _dp]
    L.ora_engine_fir.restype = C.c_size_t
    L.ora_engine_fir.argtypes = [C.c_uint, C.c_uint, _fp, C.c_size_t, C.c_int,
                                 C.c_double, C.c_double, C.c_int, _dp]
    L.ora_sdm_run_jobs.restype = C.c_int
    L.ora_dop_unpack.argtypes = [_fp, _fp, C.c_size_t]
    L.ora_boxcar_new.restype = C.c_void_p
    L.ora_boxcar_new.argtypes = [C.c_int]
    L.ora_boxcar_free.argtypes = [C.c_void_p]
    L.ora_boxcar_gain.argtypes = [C.c_void_p, _fp, _dp, C.c_size_t, C.c_double, C.c_double]
    L.ora_lowpass_design.restype = C.c_int
    L.ora_lowpass_design.argtypes = [C.c_uint, C.c_double, C.c_int, _dp]
    L.ora_lowpass_new.restype = C.c_void_p
    L.ora_lowpass_new.argtypes = [C.c_uint, C.c_double, C.c_int]
    L.ora_lowpass_free.argtypes = [C.c_void_p]
    L.ora_lowpass_taps.restype = C.c_int
    L.ora_lowpass_taps.argtypes = [C.c_void_p, _dp]
    L.ora_lowpass_process.argtypes = [C.c_void_p, _fp, _dp, C.c_size_t, C.c_double, C.c_double]
    L.ora_engine_down.restype = C.c_size_t
    L.ora_engine_down.argtypes = [C.c_void_p, C.c_void_p, _fp, C.c_size_t, C.c_double,
                                  C.c_double, C.c_int, _dp]
    L.ora_decim_new.restype = C.c_void_p
    L.ora_decim_new.argtypes = [C.c_uint, C.c_uint]
    L.ora_decim_free.argtypes = [C.c_void_p]
    L.ora_decim_process.restype = C.c_size_t
    L.ora_decim_process.argtypes = [C.c_void_p, _dp, C.c_size_t, _dp]
    L.ora_das_run_carry.restype = C.c_size_t
    L.ora_das_run_carry.argtypes = [C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_double,
                                    C.POINTER(DasCfg), C.POINTER(_dp), C.c_size_t, C.c_int,
                                    C.POINTER(_u8p), C.POINTER(C.c_int),
                                    C.POINTER(C.c_size_t), C.c_int, C.POINTER(C.c_void_p)]
    L.ora_das_run.restype = C.c_size_t
    L.ora_das_run.argtypes = [C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_double,
                              C.POINTER(DasCfg), C.POINTER(_dp), C.c_size_t, C.c_int,
                              C.POINTER(_u8p), C.POINTER(C.c_int), C.POINTER(C.c_size_t),
                              C.c_int]


def sdm(order, a, g, depth, cands, lat, state_limit=0.0) -> Sdm:
    return Sdm(oracle_lib(), order, a, g, depth, cands, lat, state_limit)


def sdm_bits(ctx: Sdm, x: np.ndarray) -> np.ndarray:
    """Run the oracle context over x and return 0/1 decision bytes."""
    x = np.ascontiguousarray(x, np.float64)
    out = np.empty(max(len(x), 1), np.uint8)
    n = ctx.L.lib.ora_sdm_process_bits(ctx.h, _ptr(x, _dp), _ptr(out, _u8p), len(x))
    return out[:n]


def segment_bits(ctx: Sdm, x: np.ndarray, discard: int) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float64)
    out = np.empty(max(len(x), 1), np.uint8)
    n = ctx.L.lib.ora_sdm_segment_bits(ctx.h, _ptr(x, _dp), _ptr(out, _u8p), len(x), discard)
    return out[:n]


def fir_design(ntaps: int, quarter: bool = False) -> np.ndarray:
    h = np.zeros(ntaps, np.float64)
    rc = oracle_lib().lib.ora_fir_design(ntaps, int(quarter), _ptr(h, _dp))
    if rc != 0:
        raise ValueError("bad tap count")
    return h


def fir_plan(fs_in: int, fs_out: int):
    fac = (C.c_int * 9)()
    nt = (C.c_int * 9)()
    s = oracle_lib().lib.ora_fir_plan(fs_in, fs_out, fac, nt)
    if s < 0:
        raise ValueError("unsupported rate pair")
    return [(fac[i], nt[i]) for i in range(s)]


def engine_fir(fs_in, fs_out, x: np.ndarray, boxcar_taps=8, g_start=1.0, g_end=1.0,
               soft_clip=True) -> np.ndarray:
    """FP64 boxcar -> FIR chain -> gain ramp -> soft clip (engine rate-conversion path)."""
    x = np.ascontiguousarray(x, np.float32)
    ratio = fs_out // fs_in
    out = np.empty(max(len(x) * ratio, 1), np.float64)
    n = oracle_lib().lib.ora_engine_fir(fs_in, fs_out, _ptr(x, _fp), len(x), boxcar_taps,
                                        g_start, g_end, int(soft_clip), _ptr(out, _dp))
    return out[:n]


def estimate_state(order, a, g, init, x, state_limit=0.0, levels=16, lib=None):
    L = lib or oracle_lib()
    aa = np.zeros(10); aa[:order] = a[:order]
    gg = np.zeros(10); gg[:order] = g[:order]
    ii = np.zeros(10); ii[:order] = init[:order]
    x = np.ascontiguousarray(x, np.float64)
    out = np.zeros(10)
    L.fn("estimate_state")(order, _ptr(aa, _dp), _ptr(gg, _dp), _ptr(ii, _dp),
                           _ptr(x, _dp), len(x), float(state_limit), levels, _ptr(out, _dp))
    return out[:order]


def dop_pack_bits(bits: np.ndarray, phase: int = 0):
    """DoP i24 frames from 0/1 decision bytes; returns (bytes, next_phase)."""
    bits = np.ascontiguousarray(bits, np.uint8)
    out = np.zeros(max(len(bits) // 16 * 3, 1), np.uint8)
    ph = oracle_lib().lib.ora_dop_pack_u8(_ptr(bits, _u8p), _ptr(out, _u8p), len(bits), phase)
    return out[: len(bits) // 16 * 3], ph


def pack_file_payload(bits: np.ndarray, fmt: str) -> np.ndarray:
    """DSF ("dsf") or DFF ("dff") payload of 0/1 decisions [nch, n]."""
    bits = np.ascontiguousarray(np.atleast_2d(bits), np.uint8)
    nch, n = bits.shape
    nbytes = (n + 7) // 8
    total = ((nbytes + 4095) // 4096) * 4096 * nch if fmt == "dsf" else nbytes * nch
    out = np.zeros(max(total, 1), np.uint8)
    fn = oracle_lib().lib.ora_pack_dsf_u8 if fmt == "dsf" else oracle_lib().lib.ora_pack_dff_u8
    fn.restype = C.c_size_t
    fn.argtypes = [_u8p, C.c_size_t, C.c_int, C.c_size_t, _u8p]
    got = fn(_ptr(bits, _u8p), n, nch, n, _ptr(out, _u8p))
    assert got == total
    return out[:total]


def ref_enc_lib():
    """The reference's offline encoder (tools/dsd_encode.c) compiled with its
    WAV I/O: file writers and input reader, or None when not built."""
    if "enc" not in _cache:
        path = os.path.join(REF_DIR, "libref_enc.so")
        if not os.path.exists(path):
            _cache["enc"] = None
        else:
            L = C.CDLL(path)
            for name in ("ref_write_dsf", "ref_write_dff"):
                getattr(L, name).argtypes = [C.c_char_p, _fp, C.c_size_t, C.c_uint32]
            L.ref_read_input.restype = C.c_longlong
            L.ref_read_input.argtypes = [C.c_char_p, _fp, C.c_size_t, C.POINTER(C.c_uint32)]
            L.ref_wav_read.restype = C.c_longlong
            L.ref_wav_read.argtypes = [C.c_char_p, _fp, C.c_size_t, C.POINTER(C.c_uint32),
                                       C.POINTER(C.c_int)]
            L.ref_wav_write.argtypes = [C.c_char_p, _fp, C.c_uint32, C.c_int, C.c_uint32]
            _cache["enc"] = L
    return _cache["enc"]


class RefPluginCfg(C.Structure):
    """ref_plugin_cfg_t of oracle/ref_plugin.c."""
    _fields_ = [("fs_out", C.c_uint), ("cands", C.c_int), ("depth", C.c_int), ("lat", C.c_int),
                ("ntf_filter", C.c_int), ("par_mode", C.c_int), ("threads", C.c_int),
                ("fir_prec", C.c_int), ("fir_mode", C.c_int), ("state_limit", C.c_float)]


def ref_plugin_lib():
    """The reference's DSP plugin core (src/dsp_plugin.c with its engine, FIR
    chain and trellis) compiled by oracle/ref_plugin.c, or None when not built."""
    if "plugin" not in _cache:
        path = os.path.join(REF_DIR, "libref_plugin.so")
        if not os.path.exists(path):
            _cache["plugin"] = None
        else:
            L = C.CDLL(path)
            L.ref_plugin_new.restype = C.c_void_p
            L.ref_plugin_new.argtypes = [C.POINTER(RefPluginCfg), C.c_int, C.c_uint]
            L.ref_plugin_process.restype = C.c_size_t
            L.ref_plugin_process.argtypes = [C.c_void_p, _fp, _u8p, C.c_size_t, C.c_int, C.c_uint]
            L.ref_plugin_fir.restype = C.c_size_t
            L.ref_plugin_fir.argtypes = [C.c_void_p, C.c_int, _dp, C.c_size_t]
            L.ref_plugin_segments.argtypes = [C.c_void_p]
            L.ref_plugin_engine_state.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 8
            L.ref_plugin_free.argtypes = [C.c_void_p]
            _cache["plugin"] = L
    return _cache["plugin"]


class RefPlugin:
    """One instance of the reference plugin on DoP input (plugin_process,
    src/dsp_plugin.c:1146-2990), trellis mode, GPU and ML absent."""

    def __init__(self, fs_in, fs_out, nch, cands, depth, lat, par_mode=-1, threads=16,
                 ntf_filter=-1, fir_prec=-1, fir_mode=-1, state_limit=-1.0):
        self.L = ref_plugin_lib()
        self.fs_in, self.fs_out, self.nch = fs_in, fs_out, nch
        cfg = RefPluginCfg(fs_out, cands, depth, lat, ntf_filter, par_mode, threads, fir_prec,
                           fir_mode, state_limit)
        self.h = self.L.ref_plugin_new(C.byref(cfg), nch, fs_in)
        if not self.h:
            raise ValueError("plugin engine init failed")

    def process(self, dop: np.ndarray) -> np.ndarray:
        """dop: interleaved DoP floats [frames, nch] -> interleaved DoP bytes."""
        dop = np.ascontiguousarray(dop, np.float32)
        frames = dop.shape[0]
        ratio = max(1, self.fs_out // self.fs_in)
        out = np.zeros(frames * ratio * 3 * self.nch + 4096, np.uint8)
        nf = self.L.ref_plugin_process(self.h, _ptr(dop, _fp), _ptr(out, _u8p), frames,
                                       self.nch, self.fs_in // 16)
        return out[: nf * 3 * self.nch]

    def fir(self) -> np.ndarray:
        """The last chunk's FIR output per channel (the DAS phase's input)."""
        rows = []
        for c in range(self.nch):
            n = self.L.ref_plugin_fir(self.h, c, None, 0)
            buf = np.zeros(max(n, 1))
            self.L.ref_plugin_fir(self.h, c, _ptr(buf, _dp), n)
            rows.append(buf[:n])
        return np.stack(rows)

    def segments(self) -> int:
        return self.L.ref_plugin_segments(self.h)

    def engine(self, ch=0) -> dict:
        """The trellis parameters the engine resolved for a channel."""
        k, d, lat, order = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        a, g = np.zeros(10), np.zeros(10)
        sl, fg = C.c_double(), C.c_float()
        mode = self.L.ref_plugin_engine_state(self.h, ch, C.byref(k), C.byref(d), C.byref(lat),
                                              C.byref(order), a.ctypes.data, g.ctypes.data,
                                              C.byref(sl), C.byref(fg))
        return dict(sdm_mode=mode, cands=k.value, depth=d.value, lat=lat.value,
                    order=order.value, a=a, g=g, state_limit=sl.value, fir_gain=fg.value)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.L.ref_plugin_free(h)
            self.h = None


def bits_pack(bits: np.ndarray) -> np.ndarray:
    bits = np.ascontiguousarray(bits, np.uint8)
    out = np.zeros(max((len(bits) + 7) // 8, 1), np.uint8)
    oracle_lib().lib.ora_bits_pack_u8(_ptr(bits, _u8p), _ptr(out, _u8p), len(bits))
    return out[: (len(bits) + 7) // 8]
