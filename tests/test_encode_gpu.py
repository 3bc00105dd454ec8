"""The offline encoder on the GPU: DSF / DFF payload packing against the
oracle's packers (whose files equal the reference's writers, see
test_dsdfile.py), and the whole encoder (WAV in -> file out) against the FIR
chain followed by the oracle's PreCorr or trellis with drain, the tool's flow
(tools/dsd_encode.c:354-574)."""
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("fmt", ["dsf", "dff"])
@pytest.mark.parametrize("nch,n", [(1, 1), (1, 70001), (2, 4096 * 8 * 3 + 5), (6, 12345)])
def test_pack_file_matches_oracle(oracle, fmt, nch, n):
    from foo_dsd_trellis_gb300 import _lib, dsdfile
    bits = (np.random.default_rng(n + nch).random((nch, n)) > 0.5).astype(np.uint8)
    code = _lib.FILE_DSF if fmt == "dsf" else _lib.FILE_DFF
    got = dsdfile.pack_payload(code, torch.from_numpy(bits).cuda()).cpu().numpy()
    assert np.array_equal(got, oracle.pack_file_payload(bits, fmt))


def _stereo_wav(path, frames, rate, seed):
    from foo_dsd_trellis_gb300 import signals
    x = signals.sine_tpdf(frames / rate, rate, 2, seed=seed)
    i16 = np.clip(np.round(x.T * 32767.0), -32768, 32767).astype("<i2")
    payload = i16.tobytes()
    fmt = struct.pack("<HHIIHH", 1, 2, rate, rate * 4, 4, 16)
    body = b"WAVE" + b"fmt " + struct.pack("<I", 16) + fmt + b"data" + struct.pack("<I", len(payload)) + payload
    path.write_bytes(b"RIFF" + struct.pack("<I", len(body)) + body)


def _fir(mono, fs_in, fs_out, gain=1.0):
    from foo_dsd_trellis_gb300.fir import FirChain
    fc = FirChain(fs_in, fs_out, boxcar_taps=0, soft_clip=False, num_channels=1)
    return fc.process(torch.from_numpy(mono).cuda(), gain, gain).cpu().numpy()[0]


def test_encode_precorr_dsf(tmp_path, oracle):
    from foo_dsd_trellis_gb300 import dsdfile, encode, ntf
    wav, out = tmp_path / "in.wav", tmp_path / "out.dsf"
    _stereo_wav(wav, 1500, 44100, 1)
    rc = encode.main(["--input", str(wav), "--dsd-rate", "5644800", "--sdm", "precorr",
                      "--ntf", "auto", "--state-limit", "12", "--gain", "0.7",
                      "--sdm-out", str(out), "--quiet"])
    assert rc == 0
    bits, fs = dsdfile.read_dsd_file(str(out))
    assert fs == 5644800 and bits.shape[0] == 1
    mono, _ = dsdfile.read_input(str(wav))
    y = _fir(mono, 44100, 5644800, 0.7)
    f = ntf.auto_select_precorr(5644800)
    want = oracle.PreCorr(f.order, np.array(f.a), np.array(f.g), 12.0).process(y)
    assert np.array_equal(bits[0, : len(want)], want)


def test_encode_trellis_dff_with_drain(tmp_path, oracle):
    from foo_dsd_trellis_gb300 import dsdfile, encode, ntf
    wav, out, fir_out = tmp_path / "in.wav", tmp_path / "out.dff", tmp_path / "fir.raw"
    _stereo_wav(wav, 300, 44100, 2)
    rc = encode.main(["--input", str(wav), "--dsd-rate", "2822400", "--ntf", "clans-6",
                      "--cands", "4", "--lat", "24", "--depth", "8", "--sdm-out", str(out),
                      "--fir-out", str(fir_out), "--quiet"])
    assert rc == 0
    bits, fs = dsdfile.read_dsd_file(str(out))
    mono, _ = dsdfile.read_input(str(wav))
    y = _fir(mono, 44100, 2822400)
    assert np.array_equal(np.fromfile(fir_out, "<f4"), y.astype(np.float32))
    f = ntf.get_filter("clans-6", 2822400)
    ctx = oracle.sdm(f.order, np.array(f.a), np.array(f.g), 8, 4, 24)
    head = ctx.process(y)
    tail = ctx.drain(len(y) - len(head))
    want = (np.concatenate([head, tail]) >= 0).astype(np.uint8)
    assert len(want) == len(y)
    assert np.array_equal(bits[0, : len(y)], want)
    assert not bits[0, len(y):].any()


def test_encode_das_keep_channels_and_float_outputs(tmp_path):
    """--das with --keep-channels equals the DAS over the FIR output of each
    channel; .wav and .raw outputs hold the same decisions as +-1 floats."""
    from foo_dsd_trellis_gb300 import dsdfile, encode, ntf
    from foo_dsd_trellis_gb300.das import DasChannels
    from foo_dsd_trellis_gb300.fir import FirChain
    wav = tmp_path / "in.wav"
    _stereo_wav(wav, 2000, 44100, 3)
    args = ["--input", str(wav), "--dsd-rate", "5644800", "--keep-channels", "--das", "32768",
            "--cands", "8", "--lat", "32", "--depth", "32", "--quiet"]
    for name in ("o.dsf", "o.wav", "o.raw"):
        assert encode.main(args + ["--sdm-out", str(tmp_path / name)]) == 0
    bits, _ = dsdfile.read_dsd_file(str(tmp_path / "o.dsf"))
    pcm, _ = dsdfile.read_input(str(wav), keep_channels=True)
    fc = FirChain(44100, 5644800, boxcar_taps=0, soft_clip=False, num_channels=2)
    y = fc.process(torch.from_numpy(pcm).cuda(), 1.0, 1.0)
    f = ntf.auto_select(5644800)
    want, _ = DasChannels(f.order, f.a, f.g, 32, 8, 32, num_channels=2).process_chunk(y, seg_len=32768)
    want = want.cpu().numpy()
    n = want.shape[1]
    assert np.array_equal(bits[:, :n], want)
    w, _ = dsdfile.wav_read(str(tmp_path / "o.wav"))
    assert np.array_equal(w, want.astype(np.float32) * 2 - 1)
    r = np.fromfile(tmp_path / "o.raw", "<f4").reshape(2, -1)
    assert np.array_equal(r, want.astype(np.float32) * 2 - 1)


def test_encode_errors(tmp_path):
    from foo_dsd_trellis_gb300 import encode
    raw = tmp_path / "x.raw"
    np.zeros(100, "<f4").tofile(raw)
    # raw input without --pcm-rate, and a rate that is not an integer multiple
    assert encode.main(["--input", str(raw), "--dsd-rate", "2822400", "--sdm-out",
                        str(tmp_path / "o.dsf"), "--quiet"]) == 1
    assert encode.main(["--input", str(raw), "--pcm-rate", "44100", "--dsd-rate", "2822401",
                        "--sdm-out", str(tmp_path / "o.dsf"), "--quiet"]) == 1
    assert encode.main(["--input", str(raw), "--dsd-rate", "2822400"]) == 1


@pytest.mark.parametrize("sdm", ["precorr", "trellis"])
def test_encode_chunked_equals_one_pass(tmp_path, sdm):
    """Chunks of 0.01 s (FIR history and SDM state carried) give the same
    file as one pass over the input."""
    from foo_dsd_trellis_gb300 import encode
    wav = tmp_path / "in.wav"
    _stereo_wav(wav, 2500, 44100, 4)
    args = ["--input", str(wav), "--dsd-rate", "2822400", "--sdm", sdm, "--cands", "4",
            "--lat", "32", "--depth", "8", "--keep-channels", "--quiet"]
    assert encode.main(args + ["--sdm-out", str(tmp_path / "a.dff"), "--chunk", "100"]) == 0
    assert encode.main(args + ["--sdm-out", str(tmp_path / "b.dff"), "--chunk", "0.01"]) == 0
    assert (tmp_path / "a.dff").read_bytes() == (tmp_path / "b.dff").read_bytes()
