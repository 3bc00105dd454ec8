"""Same-rate DSD input (DSD -> DSD re-encode): DoP unpack, the engine's
boxcar with gain ramp, and the whole pipeline, bit-exact against the oracle
(DoP unpack pinned to the reference's dop.c; boxcar restated from
src/engine.c:527-543; SDM pinned; DAS restated)."""
import numpy as np
import pytest

from signals import multitone

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dsd_stream(oracle, n, seed, order_name="clans-5", rate=2822400):
    """A DSD bitstream to re-encode: a quick trellis encode of a multitone."""
    from foo_dsd_trellis_gb300 import ntf
    f = ntf.get_filter(order_name, rate)
    ctx = oracle.sdm(f.order, np.array(f.a), np.array(f.g), 8, 4, 8)
    x = multitone(n + 8, 7 + seed) * 1.5
    return oracle.sdm_bits(ctx, x)[:n]


def test_dop_unpack(oracle):
    from foo_dsd_trellis_gb300 import _lib
    import ctypes as C
    rng = np.random.default_rng(1)
    frames, nch = 5003, 3
    bits = (rng.random((nch, 16 * frames)) > 0.5).astype(np.uint8)
    dop = np.stack([oracle.dop_float_frames(bits[c], c & 1) for c in range(nch)])
    L = _lib.load()
    h = C.c_void_p()
    assert L.dsdgpu_create(0, C.byref(h)) == 0
    d_dop = torch.from_numpy(dop).cuda()
    out = torch.empty((nch, 16 * frames + 64), dtype=torch.uint8, device="cuda")
    _lib.check(h, L.dsdgpu_dop_unpack(h, nch, C.c_void_p(d_dop.data_ptr()), d_dop.stride(0),
                                      frames, C.c_void_p(out.data_ptr()), out.stride(0)))
    got = out[:, : 16 * frames].cpu().numpy()
    for c in range(nch):
        want = (oracle.dop_unpack(dop[c]) > 0).astype(np.uint8)
        assert np.array_equal(got[c], want)
    L.dsdgpu_destroy(h)


@pytest.mark.parametrize("taps", [16, 32, 64])
def test_boxcar_streamed(oracle, taps):
    from foo_dsd_trellis_gb300 import _lib
    import ctypes as C
    rng = np.random.default_rng(taps)
    nch, n = 2, 40000
    bits = (rng.random((nch, n)) > 0.5).astype(np.uint8)
    L = _lib.load()
    h = C.c_void_p()
    assert L.dsdgpu_create(0, C.byref(h)) == 0
    _lib.check(h, L.dsdgpu_boxcar_setup(h, taps, nch))
    d_bits = torch.from_numpy(bits).cuda()
    out = torch.empty((nch, n), dtype=torch.float64, device="cuda")
    refs = [oracle.Boxcar(taps) for _ in range(nch)]
    want = [[] for _ in range(nch)]
    pos = 0
    for ln, gs, ge in ((7, 0.0, 0.9), (10000, 0.9, 0.7), (29993, 0.7, 0.7)):
        blk = d_bits[:, pos:pos + ln].contiguous()
        _lib.check(h, L.dsdgpu_boxcar_process(h, 0, nch, C.c_void_p(blk.data_ptr()), blk.stride(0),
                                              ln, C.c_void_p(out[:, pos:].data_ptr()), out.stride(0),
                                              gs, ge))
        for c in range(nch):
            want[c].append(refs[c].process(bits[c, pos:pos + ln].astype(np.float32) * 2 - 1, gs, ge))
        pos += ln
    got = out.cpu().numpy()
    for c in range(nch):
        assert np.array_equal(got[c], np.concatenate(want[c]))   # bit-exact FP64
    L.dsdgpu_destroy(h)


def test_samerate_pipeline(oracle):
    """DoP in -> unpack -> boxcar (DSD64 default 32 taps) -> DAS trellis SDM
    (CLANS-5, K = 16, depth 32, lat 32, 32,768-sample segments) -> DoP out,
    equal byte for byte to the oracle chain."""
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.pipeline import FULL_PARALLEL, OUT_DOP, Encoder
    rate, K, depth, lat, nch, gain = 2822400, 16, 32, 32, 2, 0.9
    f = ntf.get_filter("clans-5", rate)
    n = 16 * 12000
    src = np.stack([_dsd_stream(oracle, n, c) for c in range(nch)])
    dop = np.stack([oracle.dop_float_frames(src[c], 0) for c in range(nch)])
    enc = Encoder(rate, rate, nch, f, depth, K, lat, seg_len=32768, seed_mode=FULL_PARALLEL,
                  reposition=True, boxcar_taps=0, soft_clip=False, output_format=OUT_DOP)
    out = torch.empty(enc.out_capacity(dop.shape[1]) + 64, dtype=torch.uint8, device="cuda")
    ns, nb = enc.process(torch.from_numpy(dop).cuda(), out, gain, gain)
    box = np.stack([oracle.Boxcar(32).process(oracle.dop_unpack(dop[c]), gain, gain)
                    for c in range(nch)])
    bits, _, _ = oracle.das_run(f.order, np.array(f.a), np.array(f.g), depth, K, lat, 0.0, box,
                                seg_len=32768, seed_mode=0, reposition=True)
    assert bits.shape[1] == ns
    per = [oracle.dop_pack_bits(bits[c], 0)[0].reshape(-1, 3) for c in range(nch)]
    want = np.stack(per, axis=1).reshape(-1)
    assert nb == want.size
    assert np.array_equal(out[:nb].cpu().numpy(), want)


def _gpu_fir_for_dsd(dop, fs_in, fs_out, soft_clip, gs, ge, boxcar=8):
    """The FIR stage of the DSD rate-conversion pipeline from the library's
    separate entry points: unpack, then the FIR upsampling chain (boxcar 8, or
    none) or the boxcar + FP64 decimation chain (a one-tap mean for none),
    with gain and clip."""
    import ctypes as C
    from foo_dsd_trellis_gb300 import _lib
    from foo_dsd_trellis_gb300.fir import FirChain
    nch, frames = dop.shape
    n_in = 16 * frames
    d_dop = torch.from_numpy(np.ascontiguousarray(dop)).cuda()
    L = _lib.load()
    h = C.c_void_p()
    assert L.dsdgpu_create(0, C.byref(h)) == 0
    try:
        if fs_out > fs_in:
            x = torch.empty((nch, n_in), dtype=torch.float32, device="cuda")
            _lib.check(h, L.dsdgpu_dop_unpack_f32(h, nch, C.c_void_p(d_dop.data_ptr()), frames,
                                                  frames, C.c_void_p(x.data_ptr()), n_in))
            torch.cuda.synchronize()
            fc = FirChain(fs_in, fs_out, boxcar_taps=boxcar, soft_clip=soft_clip, num_channels=nch)
            y = fc.process(x, gs, ge).cpu().numpy()
            fc.close()
            return y, x.cpu().numpy()
        bits = torch.empty((nch, n_in), dtype=torch.uint8, device="cuda")
        box = torch.empty((nch, n_in), dtype=torch.float64, device="cuda")
        _lib.check(h, L.dsdgpu_dop_unpack(h, nch, C.c_void_p(d_dop.data_ptr()), frames, frames,
                                          C.c_void_p(bits.data_ptr()), n_in))
        _lib.check(h, L.dsdgpu_boxcar_setup(h, max(1, boxcar), nch))
        _lib.check(h, L.dsdgpu_boxcar_process(h, 0, nch, C.c_void_p(bits.data_ptr()), n_in, n_in,
                                              C.c_void_p(box.data_ptr()), n_in, 1.0, 1.0))
        _lib.check(h, L.dsdgpu_decim_setup(h, fs_in, fs_out, nch))
        out = torch.empty((nch, n_in), dtype=torch.float64, device="cuda")
        n = C.c_size_t()
        _lib.check(h, L.dsdgpu_decim_process_f64(h, nch, C.c_void_p(box.data_ptr()), n_in, n_in,
                                                 C.c_void_p(out.data_ptr()), n_in, gs, ge,
                                                 int(soft_clip), C.byref(n)))
        return out[:, : n.value].cpu().numpy(), bits.cpu().numpy().astype(np.float32) * 2 - 1
    finally:
        L.dsdgpu_destroy(h)


@pytest.mark.parametrize("fs_in,fs_out,mode", [(2822400, 5644800, "precorr"),
                                               (2822400, 11289600, "trellis"),
                                               (5644800, 2822400, "trellis"),
                                               (11289600, 5644800, "precorr")])
def test_dsd_rate_conversion_pipeline(oracle, fs_in, fs_out, mode):
    """DSD -> DSD at another rate, the engine's rate-conversion branch with DSD
    input (src/engine.c:600-729): DoP unpack, boxcar 8, FIR up (FP32 polyphase,
    FP64 epilogue) or FP64 decimation down, gain ramp, soft clip unless
    PreCorr, then the DAS trellis or PreCorr and packing.  The FIR stage is
    checked against the oracle's FP64 restatement (1e-6 of full scale up, as
    the PCM chain; 1e-12 down, FP64 throughout) and the pipeline's decisions
    equal the oracle's SDM on that stage's output byte for byte."""
    from foo_dsd_trellis_gb300 import _lib, ntf
    from foo_dsd_trellis_gb300.pipeline import FULL_PARALLEL, OUT_BITS, Encoder
    nch, K, depth, lat, ge = 2, 2, 4, 32, float(np.float32(0.708))
    frames = 6000 if fs_out > fs_in else 12000
    src = np.stack([_dsd_stream(oracle, 16 * frames, 5 + c, "clans-5", fs_in) for c in range(nch)])
    dop = np.stack([oracle.dop_float_frames(src[c], 0) for c in range(nch)])
    precorr = mode == "precorr"
    f = ntf.auto_select_precorr(fs_out) if precorr else ntf.get_filter("clans-6", fs_out)
    clip = not precorr
    fir, x = _gpu_fir_for_dsd(dop, fs_in, fs_out, clip, 0.0, ge)
    if fs_out > fs_in:
        want_fir = np.stack([oracle.engine_fir(fs_in, fs_out, x[c], 8, ge, ge, clip) for c in range(nch)])
        tol = 1e-6
    else:
        want_fir = np.stack([oracle.engine_down(oracle.Boxcar(8), oracle.Decimator(fs_in, fs_out),
                                                x[c], 0.0, ge, clip) for c in range(nch)])
        tol = 1e-12
    assert fir.shape == want_fir.shape
    assert np.max(np.abs(fir - want_fir)) <= tol * np.max(np.abs(want_fir))
    enc = Encoder(fs_in, fs_out, nch, f, depth, K, lat, seg_len=32768, seed_mode=FULL_PARALLEL,
                  reposition=True, boxcar_taps=8, soft_clip=True, output_format=OUT_BITS,
                  sdm_mode=_lib.SDM_PRECORR if precorr else _lib.SDM_TRELLIS)
    n_fir = fir.shape[1]
    out = torch.empty((nch, n_fir + 256), dtype=torch.uint8, device="cuda")
    ns, _ = enc.process(torch.from_numpy(dop).cuda(), out, 0.0, ge)
    got = out[:, :ns].cpu().numpy()
    if precorr:
        want = np.stack([oracle.PreCorr(f.order, np.array(f.a), np.array(f.g), 0.0).process(fir[c])
                         for c in range(nch)])
    else:
        want, _, _ = oracle.das_run(f.order, np.array(f.a), np.array(f.g), depth, K, lat, 0.0, fir,
                                    seg_len=32768, seed_mode=0, reposition=True)
    assert got.shape == want.shape
    assert np.array_equal(got, want)
    enc.close()



@pytest.mark.parametrize("fs_in,fs_out", [(2822400, 11289600), (11289600, 5644800)],
                         ids=["up4", "down2"])
def test_dsd_rate_conversion_das_glue(oracle, fs_in, fs_out):
    """The plugin's DAS path for DSD input at another rate runs the engine's FIR
    phase without the boxcar and the soft clip (engine_process_fir_gain,
    src/engine.c:789-900; pinned to the reference's engine.c on the CPU): the
    pipeline with boxcar_taps 0 and soft_clip 0 equals that FIR stage (1e-6 of
    full scale up, 1e-12 down against the oracle's restatement) followed by the
    oracle's DAS, byte for byte."""
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.pipeline import FULL_PARALLEL, OUT_BITS, Encoder
    nch, K, depth, lat, ge = 2, 2, 4, 32, float(np.float32(0.708))
    frames = 6000 if fs_out > fs_in else 12000
    src = np.stack([_dsd_stream(oracle, 16 * frames, 9 + c, "clans-5", fs_in) for c in range(nch)])
    dop = np.stack([oracle.dop_float_frames(src[c], 0) for c in range(nch)])
    f = ntf.get_filter("clans-6", fs_out)
    fir, x = _gpu_fir_for_dsd(dop, fs_in, fs_out, False, ge, ge, boxcar=0)
    if fs_out > fs_in:
        want_fir = np.stack([oracle.engine_fir(fs_in, fs_out, x[c], 0, ge, ge, False) for c in range(nch)])
        tol = 1e-6
    else:
        want_fir = np.stack([oracle.engine_down(oracle.Boxcar(1), oracle.Decimator(fs_in, fs_out),
                                                x[c], ge, ge, False) for c in range(nch)])
        tol = 1e-12
    assert fir.shape == want_fir.shape
    assert np.max(np.abs(fir - want_fir)) <= tol * np.max(np.abs(want_fir))
    enc = Encoder(fs_in, fs_out, nch, f, depth, K, lat, seg_len=32768, seed_mode=FULL_PARALLEL,
                  reposition=True, boxcar_taps=0, soft_clip=False, output_format=OUT_BITS)
    out = torch.empty((nch, fir.shape[1] + 256), dtype=torch.uint8, device="cuda")
    ns, _ = enc.process(torch.from_numpy(dop).cuda(), out, ge, ge)
    want, _, _ = oracle.das_run(f.order, np.array(f.a), np.array(f.g), depth, K, lat, 0.0, fir,
                                seg_len=32768, seed_mode=0, reposition=True)
    assert np.array_equal(out[:, :ns].cpu().numpy(), want)
    enc.close()
