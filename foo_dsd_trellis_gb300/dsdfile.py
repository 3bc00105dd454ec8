"""File formats of the offline encoder: WAV in, DSF / DSDIFF / WAV / raw out.

Mirrors the reference's tools/dsd_encode.c (read_input :118-162, writers
:164-312) and src/wav_io.c (wav_read :43-152, wav_write :154-186):

* `wav_read` parses RIFF/WAVE the way wav_read does (chunk scan up to the
  first "data" chunk, PCM 16/24/32-bit or IEEE float 32, the same integer to
  float conversions) and raises ValueError where it returns -1;
* `read_input` is the tool's input reader: a WAV mixed to mono in float32
  (sum over channels from 0, then divided by the channel count), else raw
  float32 samples;
* DSF / DFF files are a header from libdsdgpu (`dsdgpu_file_header`, host
  code) and a payload packed on the device (`dsdgpu_pack_file`).
"""
from __future__ import annotations

import ctypes as C
import struct

import numpy as np
import torch

from . import _lib

_WAV_PCM, _WAV_FLOAT = 1, 3


def wav_read(path: str) -> tuple[np.ndarray, int]:
    """Returns (float32 [channels, frames], sample rate)."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < 12 or data[0:4] != b"RIFF" or data[8:12] != b"WAVE":
        raise ValueError("not a RIFF/WAVE file")
    pos = 12
    fmt = None
    data_off = data_size = 0
    while pos + 8 <= len(data):
        cid, size = data[pos:pos + 4], struct.unpack_from("<I", data, pos + 4)[0]
        pos += 8
        if cid == b"fmt ":
            raw = data[pos:pos + min(size, 16)].ljust(16, b"\0")
            if pos + min(size, 16) > len(data):
                break
            fmt = struct.unpack("<HHIIHH", raw)
            pos += size
        elif cid == b"data":
            data_off, data_size = pos, size
            break
        else:
            pos += size
    if fmt is None or data_off == 0 or data_size == 0:
        raise ValueError("no fmt or data chunk")
    format_tag, channels, rate, _, _, bits = fmt
    if format_tag not in (_WAV_PCM, _WAV_FLOAT) or channels == 0 or bits == 0:
        raise ValueError("unsupported WAV format")
    bps = bits // 8
    frame = bps * channels
    if frame == 0:
        raise ValueError("zero frame size")
    frames = data_size // frame
    if data_off + data_size > len(data):
        raise ValueError("truncated data chunk")
    raw = np.frombuffer(data, np.uint8, frames * frame, data_off)
    if format_tag == _WAV_FLOAT and bps == 4:
        x = raw.view("<f4").astype(np.float32)
    elif format_tag == _WAV_PCM and bps == 2:
        x = raw.view("<i2").astype(np.float32) / np.float32(32768.0)
    elif format_tag == _WAV_PCM and bps == 3:
        b = raw.reshape(-1, 3).astype(np.int32)
        v = b[:, 0] | (b[:, 1] << 8) | (b[:, 2] << 16)
        v = np.where(v & 0x800000, v - (1 << 24), v).astype(np.int32)
        x = v.astype(np.float32) / np.float32(8388608.0)
    elif format_tag == _WAV_PCM and bps == 4:
        x = (raw.view("<i4").astype(np.float64) / 2147483648.0).astype(np.float32)
    else:
        raise ValueError("unsupported sample format")
    return np.ascontiguousarray(x.reshape(frames, channels).T), int(rate)


def wav_write(path: str, samples: np.ndarray, rate: int) -> None:
    """32-bit float WAV of float32 [channels, frames] (wav_write's layout)."""
    x = np.ascontiguousarray(np.atleast_2d(samples).T, "<f4")
    frames, ch = x.shape
    data_size = frames * ch * 4
    hdr = b"RIFF" + struct.pack("<I", 36 + data_size) + b"WAVE"
    hdr += b"fmt " + struct.pack("<IHHIIHH", 16, _WAV_FLOAT, ch, rate, rate * ch * 4, ch * 4, 32)
    hdr += b"data" + struct.pack("<I", data_size)
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(x.tobytes())


def read_input(path: str, keep_channels: bool = False) -> tuple[np.ndarray, int]:
    """The encoder's input: (float32 [channels, frames], rate).  A WAV is mixed
    to mono unless keep_channels; anything else is raw float32 mono with rate
    0 (the caller supplies it)."""
    try:
        x, rate = wav_read(path)
    except ValueError:
        return np.fromfile(path, "<f4").astype(np.float32)[None, :], 0
    if keep_channels or x.shape[0] == 1:
        return x, rate
    s = np.zeros(x.shape[1], np.float32)
    for c in range(x.shape[0]):
        s = s + x[c]
    return (s / np.float32(x.shape[0]))[None, :], rate


def file_header(fmt: int, nch: int, fs: int, samples: int) -> tuple[bytes, int]:
    """(header bytes, payload size) of a DSF / DFF file (host only)."""
    L = _lib.load()
    buf = (C.c_uint8 * 256)()
    n = C.c_size_t()
    pay = C.c_uint64()
    rc = L.dsdgpu_file_header(fmt, nch, fs, samples, buf, 256, C.byref(n), C.byref(pay))
    if rc != _lib.OK:
        raise _lib.DsdGpuError(rc, "dsdgpu_file_header failed")
    return bytes(buf[: n.value]), pay.value


def pack_payload(fmt: int, bits: torch.Tensor, device: int = 0) -> torch.Tensor:
    """Decision bytes [nch, n] (uint8, CUDA) -> the file's payload on the device."""
    L = _lib.load()
    bits = bits.contiguous()
    nch, n = bits.shape
    _, pay = file_header(fmt, nch, 2822400, n)
    out = torch.empty(max(pay, 1), dtype=torch.uint8, device=bits.device)
    h = C.c_void_p()
    rc = L.dsdgpu_create(device, C.byref(h))
    if rc != _lib.OK:
        raise _lib.DsdGpuError(rc, "dsdgpu_create failed")
    try:
        got = C.c_uint64()
        torch.cuda.current_stream().synchronize()
        _lib.check(h, L.dsdgpu_pack_file(h, fmt, nch, C.c_void_p(bits.data_ptr()), n, n,
                                         C.c_void_p(out.data_ptr()), C.byref(got)))
    finally:
        L.dsdgpu_destroy(h)
    return out[:pay]


def write_dsd_file(path: str, fmt: int, bits: torch.Tensor, fs: int, device: int = 0) -> None:
    """DSF / DFF file of decision bytes [nch, n] at fs Hz."""
    nch, n = bits.shape
    hdr, _ = file_header(fmt, nch, fs, n)
    payload = pack_payload(fmt, bits, device).cpu().numpy()
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(payload.tobytes())


def read_dsd_file(path: str) -> tuple[np.ndarray, int]:
    """Decisions [nch, n] and rate of a DSF or DFF file in the layouts above
    (used to check written files)."""
    with open(path, "rb") as f:
        d = f.read()
    if d[:4] == b"DSD ":
        ch = struct.unpack_from("<I", d, 28 + 24)[0]
        fs = struct.unpack_from("<I", d, 28 + 28)[0]
        n = struct.unpack_from("<Q", d, 28 + 36)[0]
        blk = struct.unpack_from("<I", d, 28 + 44)[0]
        pay = np.frombuffer(d, np.uint8, offset=92)
        blocks = pay.reshape(-1, ch, blk).transpose(1, 0, 2).reshape(ch, -1)
        bits = np.unpackbits(blocks, axis=1, bitorder="little")[:, :n]
        return bits, fs
    if d[:4] == b"FRM8":
        pos, fs, ch = 16, 0, 0
        while pos + 12 <= len(d):
            cid, size = d[pos:pos + 4], struct.unpack_from(">Q", d, pos + 4)[0]
            if cid == b"PROP":
                q = pos + 16
                while q < pos + 12 + size:
                    sid, ssz = d[q:q + 4], struct.unpack_from(">Q", d, q + 4)[0]
                    if sid == b"FS  ":
                        fs = struct.unpack_from(">I", d, q + 12)[0]
                    elif sid == b"CHNL":
                        ch = struct.unpack_from(">H", d, q + 12)[0]
                    q += 12 + ssz
            elif cid == b"DSD ":
                pay = np.frombuffer(d, np.uint8, size, pos + 12)
                bits = np.unpackbits(pay.reshape(-1, ch).T, axis=1)
                return bits, fs
            pos += 12 + size
    raise ValueError("not a DSF or DFF file")
