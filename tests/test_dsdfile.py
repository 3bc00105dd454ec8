"""Offline-encoder file formats, on the CPU: DSF / DFF files made of the
library's header (host code) and the oracle's payload packers equal the
reference's own write_dsf / write_dff byte for byte (tools/dsd_encode.c,
compiled from the reference tree into oracle/_ref); the WAV reader, the
encoder's input reader and the WAV writer equal src/wav_io.c and the tool's
read_input.  Multichannel layouts (no reference counterpart) round-trip."""
import ctypes as C
import os
import struct

import numpy as np
import pytest


@pytest.fixture(scope="module")
def enc(oracle):
    L = oracle.ref_enc_lib()
    if L is None:
        pytest.skip("reference build (oracle/_ref) not present")
    return L


@pytest.fixture(scope="module")
def dsdfile():
    from foo_dsd_trellis_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build_library()
    from foo_dsd_trellis_gb300 import dsdfile as D
    return D


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


@pytest.mark.parametrize("fmt", ["dsf", "dff"])
@pytest.mark.parametrize("n", [1, 7, 8, 9, 1000, 32768, 32768 * 8 + 5, 100003])
def test_mono_file_equals_reference_writer(tmp_path, oracle, enc, dsdfile, fmt, n):
    from foo_dsd_trellis_gb300 import _lib
    rng = np.random.default_rng(n)
    bits = (rng.random(n) > 0.5).astype(np.uint8)
    rate = 5644800 if n % 2 else 2822400
    ref_path = str(tmp_path / f"ref.{fmt}")
    f = np.where(bits > 0, 1.0, -1.0).astype(np.float32)
    writer = enc.ref_write_dsf if fmt == "dsf" else enc.ref_write_dff
    assert writer(ref_path.encode(), _fp(f), n, rate) == 0
    code = _lib.FILE_DSF if fmt == "dsf" else _lib.FILE_DFF
    hdr, pay = dsdfile.file_header(code, 1, rate, n)
    body = oracle.pack_file_payload(bits[None, :], fmt)
    assert len(body) == pay
    mine = hdr + body.tobytes()
    ref = open(ref_path, "rb").read()
    assert len(mine) == len(ref)
    assert mine == ref


@pytest.mark.parametrize("fmt", ["dsf", "dff"])
@pytest.mark.parametrize("nch", [2, 3, 6])
def test_multichannel_layout_round_trip(tmp_path, oracle, dsdfile, fmt, nch):
    from foo_dsd_trellis_gb300 import _lib
    n = 4096 * 8 * 2 + 13
    bits = (np.random.default_rng(nch).random((nch, n)) > 0.5).astype(np.uint8)
    code = _lib.FILE_DSF if fmt == "dsf" else _lib.FILE_DFF
    hdr, pay = dsdfile.file_header(code, nch, 11289600, n)
    body = oracle.pack_file_payload(bits, fmt)
    assert len(body) == pay
    p = tmp_path / f"m.{fmt}"
    p.write_bytes(hdr + body.tobytes())
    got, fs = dsdfile.read_dsd_file(str(p))
    assert fs == 11289600
    assert np.array_equal(got[:, :n], bits)
    if fmt == "dsf":
        assert struct.unpack_from("<Q", hdr, 12)[0] == len(hdr) + pay    # total file size
        assert struct.unpack_from("<I", hdr, 28 + 20)[0] == {2: 2, 3: 3, 6: 7}[nch]
    else:
        assert struct.unpack_from(">Q", hdr, 4)[0] == len(hdr) + pay - 12  # FRM8 payload


def test_file_header_rejects(dsdfile):
    from foo_dsd_trellis_gb300 import _lib
    with pytest.raises(_lib.DsdGpuError):
        dsdfile.file_header(_lib.FILE_DSF, 7, 2822400, 10)
    with pytest.raises(_lib.DsdGpuError):
        dsdfile.file_header(9, 1, 2822400, 10)


def _wav_bytes(fmt_tag, bits, ch, rate, payload, extra_fmt=b"", lead=b""):
    bps = bits // 8
    fmt = struct.pack("<HHIIHH", fmt_tag, ch, rate, rate * ch * bps, ch * bps, bits) + extra_fmt
    body = b"WAVE" + lead + b"fmt " + struct.pack("<I", len(fmt)) + fmt
    body += b"data" + struct.pack("<I", len(payload)) + payload
    return b"RIFF" + struct.pack("<I", len(body)) + body


def _cases():
    rng = np.random.default_rng(7)
    out = []
    for ch in (1, 2, 3):
        n = 1001
        i16 = rng.integers(-32768, 32768, n * ch).astype("<i2")
        out.append(("pcm16", _wav_bytes(1, 16, ch, 44100, i16.tobytes())))
        i24 = rng.integers(-(1 << 23), 1 << 23, n * ch)
        b24 = np.stack([i24 & 0xFF, (i24 >> 8) & 0xFF, (i24 >> 16) & 0xFF], 1).astype(np.uint8)
        out.append(("pcm24", _wav_bytes(1, 24, ch, 48000, b24.tobytes(), extra_fmt=b"\0\0",
                                        lead=b"LIST" + struct.pack("<I", 6) + b"abcdef")))
        i32 = rng.integers(-(1 << 31), 1 << 31, n * ch).astype("<i4")
        out.append(("pcm32", _wav_bytes(1, 32, ch, 96000, i32.tobytes())))
        f32 = (rng.standard_normal(n * ch) * 0.3).astype("<f4")
        f32[:4] = [-0.0, 0.0, 1.0, -1.0][: 4]
        out.append(("float", _wav_bytes(3, 32, ch, 88200, f32.tobytes())))
    return out


@pytest.mark.parametrize("k", range(12))
def test_wav_read_and_input_equal_reference(tmp_path, enc, dsdfile, k):
    name, data = _cases()[k]
    p = tmp_path / f"{name}.wav"
    p.write_bytes(data)
    x, rate = dsdfile.wav_read(str(p))
    ch, n = x.shape
    buf = np.zeros(ch * n + 16, np.float32)
    r, c = C.c_uint32(), C.c_int()
    frames = enc.ref_wav_read(str(p).encode(), _fp(buf), len(buf), C.byref(r), C.byref(c))
    assert (frames, r.value, c.value) == (n, rate, ch)
    assert np.array_equal(x.T.reshape(-1).view(np.uint32), buf[: ch * n].view(np.uint32))
    mono, rate2 = dsdfile.read_input(str(p))
    got = enc.ref_read_input(str(p).encode(), _fp(buf), len(buf), C.byref(r))
    assert got == n and r.value == rate2 == rate
    assert np.array_equal(mono[0].view(np.uint32), buf[:n].view(np.uint32))


def test_raw_input_and_wav_write_equal_reference(tmp_path, enc, dsdfile):
    raw = (np.random.default_rng(3).standard_normal(777) * 0.2).astype("<f4")
    p = tmp_path / "in.raw"
    raw.tofile(p)
    mono, rate = dsdfile.read_input(str(p))
    buf = np.zeros(800, np.float32)
    r = C.c_uint32()
    assert enc.ref_read_input(str(p).encode(), _fp(buf), len(buf), C.byref(r)) == 777
    assert rate == 0 and r.value == 0
    assert np.array_equal(mono[0], buf[:777])
    x = (np.random.default_rng(4).standard_normal((2, 333)) * 0.5).astype(np.float32)
    mine, ref = tmp_path / "a.wav", tmp_path / "b.wav"
    dsdfile.wav_write(str(mine), x, 5644800)
    inter = np.ascontiguousarray(x.T.reshape(-1))
    assert enc.ref_wav_write(str(ref).encode(), _fp(inter), 333, 2, 5644800) == 0
    assert mine.read_bytes() == ref.read_bytes()
