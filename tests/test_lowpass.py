"""Same-rate FIR lowpass (the engine's FIR_MODE_FIR branch, reference
src/engine.c:505-523, fir_lowpass_init_ex / fir_lowpass_process
src/fir.c:795-872).  The reference's fir.c needs Intel IPP and does not build
here, so the design and filtering are restated (oracle/dsd_oracle.c) and
checked on their own terms: the library's host-side design equals the
oracle's bit for bit, the restatement equals a direct-form FP64 convolution
to rounding, streaming equals one pass, and on the GPU the kernel equals the
restatement bit for bit (tests/test_lowpass.py::test_lowpass_gpu_*)."""
import ctypes as C

import numpy as np
import pytest

CASES = [(2822400, 50000.0, 127), (5644800, 50000.0, 127), (22579200, 50000.0, 127),
         (2822400, 30000.0, 33), (2822400, 80000.0, 2), (5644800, 50000.0, 128),
         (2822400, 50000.0, 400), (96000, 60000.0, 63), (2822400, 20000.0, 255)]


@pytest.mark.parametrize("fs,cut,nt", CASES)
def test_library_design_equals_oracle(oracle, fs, cut, nt):
    from foo_dsd_trellis_gb300 import _lib
    L = _lib.load()
    h = np.zeros(256, np.float64)
    n = C.c_int()
    assert L.dsdgpu_lowpass_design(fs, cut, nt, C.c_void_p(h.ctypes.data), 256, C.byref(n)) == 0
    want = oracle.lowpass_design(fs, cut, nt)
    assert n.value == len(want)
    assert np.array_equal(h[: n.value].view(np.uint64), want.view(np.uint64))


def test_design_rules(oracle):
    # ntaps clamped to 3..255 and made odd; fc capped at 0.5
    assert len(oracle.lowpass_design(2822400, 50000.0, 2)) == 3
    assert len(oracle.lowpass_design(2822400, 50000.0, 128)) == 129
    assert len(oracle.lowpass_design(2822400, 50000.0, 1000)) == 255
    h = oracle.lowpass_design(96000, 60000.0, 63)         # cutoff above fs / 2
    assert np.allclose(h, oracle.lowpass_design(96000, 48000.0, 63), rtol=0, atol=0)
    for fs in (2822400, 5644800, 11289600, 22579200):
        h = oracle.lowpass_design(fs, 50000.0, 127)
        assert abs(h.sum() - 1.0) < 1e-14                    # normalised to unit sum
        assert np.allclose(h, h[::-1], rtol=1e-12, atol=0)    # linear phase (to rounding)
        w = np.fft.rfft(h, 1 << 16)
        f = np.arange(len(w)) * fs / (1 << 16)
        # 50 kHz design: flat at DC, deep stopband well above the cutoff
        assert abs(abs(w[0]) - 1.0) < 1e-12
        assert 20 * np.log10(np.abs(w[f > 50000.0 + 0.12 * fs]).max()) < -80


def test_restatement_is_the_convolution(oracle):
    """The grouped summation order equals y[i] = sum_k h[k] x[i-k] with zeros
    before the first sample, up to FP64 rounding, and streaming with the
    delay line carried equals one pass bit for bit."""
    rng = np.random.default_rng(3)
    x = np.where(rng.random(20000) > 0.5, 1.0, -1.0).astype(np.float32)
    for fs, cut, nt in ((2822400, 50000.0, 127), (5644800, 40000.0, 61), (2822400, 20000.0, 255)):
        lp = oracle.Lowpass(fs, cut, nt)
        h = lp.taps()
        one = lp.process(x, 0.8, 0.8)
        want = np.convolve(x.astype(np.float64), h)[: len(x)] * 0.8
        assert np.max(np.abs(one - want)) < 1e-14
        lp2 = oracle.Lowpass(fs, cut, nt)
        parts, pos = [], 0
        for ln in (1, 5, 200, 7, 4096, len(x) - 4309):
            parts.append(lp2.process(x[pos:pos + ln], 0.8, 0.8))
            pos += ln
        assert pos == len(x)
        assert np.array_equal(np.concatenate(parts), one)


def _ctx():
    from foo_dsd_trellis_gb300 import _lib
    L = _lib.load()
    h = C.c_void_p()
    assert L.dsdgpu_create(0, C.byref(h)) == 0
    return L, h


@pytest.mark.gpu
@pytest.mark.parametrize("fs,cut,nt", [(2822400, 50000.0, 127), (5644800, 50000.0, 127),
                                       (2822400, 80000.0, 3), (2822400, 30000.0, 33),
                                       (2822400, 20000.0, 255)])
def test_lowpass_gpu_streamed(oracle, fs, cut, nt):
    torch = pytest.importorskip("torch")
    from foo_dsd_trellis_gb300 import _lib
    rng = np.random.default_rng(nt)
    nch, n = 3, 60000
    bits = (rng.random((nch, n)) > 0.5).astype(np.uint8)
    L, h = _ctx()
    _lib.check(h, L.dsdgpu_lowpass_setup(h, fs, cut, nt, nch))
    got_taps = np.zeros(256)
    cnt = C.c_int()
    _lib.check(h, L.dsdgpu_lowpass_taps(h, C.c_void_p(got_taps.ctypes.data), 256, C.byref(cnt)))
    refs = [oracle.Lowpass(fs, cut, nt) for _ in range(nch)]
    assert np.array_equal(got_taps[: cnt.value], refs[0].taps())
    d_bits = torch.from_numpy(bits).cuda()
    out = torch.empty((nch, n), dtype=torch.float64, device="cuda")
    want = [[] for _ in range(nch)]
    pos = 0
    # blocks shorter than the window, one sample, tile-sized and ragged
    for ln, gs, ge in ((7, 0.0, 0.9), (1, 0.9, 0.9), (100, 0.9, 0.7), (256, 0.7, 0.7),
                       (10000, 0.7, 1.1), (n - 10364, 1.1, 1.1)):
        blk = d_bits[:, pos:pos + ln].contiguous()
        _lib.check(h, L.dsdgpu_lowpass_process(h, 0, nch, C.c_void_p(blk.data_ptr()), blk.stride(0),
                                               ln, C.c_void_p(out[:, pos:].data_ptr()), out.stride(0),
                                               gs, ge))
        for c in range(nch):
            want[c].append(refs[c].process(bits[c, pos:pos + ln].astype(np.float32) * 2 - 1, gs, ge))
        pos += ln
    got = out.cpu().numpy()
    for c in range(nch):
        assert np.array_equal(got[c], np.concatenate(want[c]))   # bit-exact FP64
    L.dsdgpu_destroy(h)


@pytest.mark.gpu
def test_lowpass_gpu_channels_reset_errors(oracle):
    torch = pytest.importorskip("torch")
    from foo_dsd_trellis_gb300 import _lib
    rng = np.random.default_rng(9)
    nch, n = 4, 5000
    bits = (rng.random((nch, n)) > 0.5).astype(np.uint8)
    L, h = _ctx()
    _lib.check(h, L.dsdgpu_lowpass_setup(h, 5644800, 50000.0, 127, nch))
    d_bits = torch.from_numpy(bits).cuda()
    out = torch.zeros((nch, n), dtype=torch.float64, device="cuda")
    # channels 1..2 only, then channel 3 alone; channel 0 untouched
    _lib.check(h, L.dsdgpu_lowpass_process(h, 1, 2, C.c_void_p(d_bits[1].data_ptr()), n, 3000,
                                           C.c_void_p(out[1].data_ptr()), n, 1.0, 1.0))
    _lib.check(h, L.dsdgpu_lowpass_process(h, 3, 1, C.c_void_p(d_bits[3].data_ptr()), n, n,
                                           C.c_void_p(out[3].data_ptr()), n, 1.0, 1.0))
    got = out.cpu().numpy()
    assert not got[0].any()
    for c in (1, 2):
        want = oracle.Lowpass(5644800).process(bits[c, :3000].astype(np.float32) * 2 - 1, 1.0, 1.0)
        assert np.array_equal(got[c, :3000], want)
    # reset: the next block starts from a zero delay line again
    _lib.check(h, L.dsdgpu_lowpass_reset(h))
    _lib.check(h, L.dsdgpu_lowpass_process(h, 3, 1, C.c_void_p(d_bits[3].data_ptr()), n, 500,
                                           C.c_void_p(out[3].data_ptr()), n, 1.0, 1.0))
    want = oracle.Lowpass(5644800).process(bits[3, :500].astype(np.float32) * 2 - 1, 1.0, 1.0)
    assert np.array_equal(out[3, :500].cpu().numpy(), want)
    assert L.dsdgpu_lowpass_process(h, 3, 2, C.c_void_p(d_bits.data_ptr()), n, 10,
                                    C.c_void_p(out.data_ptr()), n, 1.0, 1.0) == _lib.ERR_ARG
    assert L.dsdgpu_lowpass_process(h, 0, 1, None, n, 10, C.c_void_p(out.data_ptr()), n,
                                    1.0, 1.0) == _lib.ERR_ARG
    assert L.dsdgpu_lowpass_process(h, 0, 1, C.c_void_p(d_bits.data_ptr()), n, 0, None, n,
                                    1.0, 1.0) == _lib.OK
    L.dsdgpu_destroy(h)
    L, h = _ctx()
    assert L.dsdgpu_lowpass_reset(h) == _lib.ERR_STATE
    assert L.dsdgpu_lowpass_setup(h, 0, 50000.0, 127, 1) == _lib.ERR_ARG
    L.dsdgpu_destroy(h)


@pytest.mark.gpu
@pytest.mark.parametrize("sdm_mode", ["trellis", "precorr"])
def test_samerate_lowpass_pipeline(oracle, sdm_mode):
    """DoP in -> unpack -> FIR lowpass -> DAS trellis SDM (one chunk) or
    PreCorr (two chunks, delay line and SDM state carried) -> DoP out, equal
    byte for byte to the oracle chain, with a gain ramp."""
    torch = pytest.importorskip("torch")
    from foo_dsd_trellis_gb300 import _lib, ntf
    from foo_dsd_trellis_gb300.pipeline import FULL_PARALLEL, OUT_DOP, Encoder
    from test_dsd_gpu import _dsd_stream
    rate, K, depth, lat, nch = 5644800, 8, 16, 32, 2
    f = ntf.get_filter("clans-6", rate)
    n = 16 * 9000
    src = np.stack([_dsd_stream(oracle, n, c, "clans-5", 2822400) for c in range(nch)])
    dop = np.stack([oracle.dop_float_frames(src[c], 0) for c in range(nch)])
    precorr = sdm_mode == "precorr"
    enc = Encoder(rate, rate, nch, f, depth, K, lat, seg_len=32768, seed_mode=FULL_PARALLEL,
                  reposition=True, soft_clip=False, output_format=OUT_DOP,
                  sdm_mode=_lib.SDM_PRECORR if precorr else _lib.SDM_TRELLIS,
                  samerate_filter=_lib.SAMERATE_LOWPASS)
    lps = [oracle.Lowpass(rate) for _ in range(nch)]
    pcs = [oracle.PreCorr(f.order, np.array(f.a), np.array(f.g), 0.0) for _ in range(nch)]
    half = dop.shape[1] // 2
    chunks = ((0, half, 0.0, 0.9), (half, dop.shape[1], 0.9, 0.8)) if precorr else \
        ((0, dop.shape[1], 0.0, 0.9),)
    phase = 0
    for lo, hi, gs, ge in chunks:
        chunk = np.ascontiguousarray(dop[:, lo:hi])
        out = torch.empty(enc.out_capacity(chunk.shape[1]) + 64, dtype=torch.uint8, device="cuda")
        ns, nb = enc.process(torch.from_numpy(chunk).cuda(), out, gs, ge)
        fir = np.stack([lps[c].process(oracle.dop_unpack(chunk[c]), gs, ge) for c in range(nch)])
        if precorr:
            bits = np.stack([pcs[c].process(fir[c]) for c in range(nch)])
        else:
            bits, _, _ = oracle.das_run(f.order, np.array(f.a), np.array(f.g), depth, K, lat, 0.0,
                                        fir, seg_len=32768, seed_mode=0, reposition=True)
        assert bits.shape[1] == ns
        packed = [oracle.dop_pack_bits(bits[c], phase) for c in range(nch)]
        phase = packed[0][1]
        want = np.stack([p[0].reshape(-1, 3) for p in packed], axis=1).reshape(-1)
        assert nb == want.size
        assert np.array_equal(out[:nb].cpu().numpy(), want)
    enc.close()
