"""DSD -> PCM decimation (the reference's FIR-only engine branch): the GPU
chain against the oracle's FP64 restatement of the half-band /2 stages with
IPP FIRMR semantics (streamed, odd block lengths), and the whole DoP -> PCM
pipeline's SINAD on a DSD128 tone, which the reference's README table puts
above 120 dB for DSD128 -> 44.1 kHz (README.md:589-600)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("fs_in,fs_out", [(2822400, 44100), (5644800, 176400), (11289600, 88200)])
def test_decim_matches_oracle(oracle, fs_in, fs_out):
    from foo_dsd_trellis_gb300 import _lib
    rng = np.random.default_rng(fs_in // fs_out)
    nch, n = 2, 300000
    bits = (rng.random((nch, n)) > 0.5).astype(np.uint8)
    L = _lib.load()
    h = C.c_void_p()
    assert L.dsdgpu_create(0, C.byref(h)) == 0
    _lib.check(h, L.dsdgpu_decim_setup(h, fs_in, fs_out, nch))
    refs = [oracle.Decimator(fs_in, fs_out) for _ in range(nch)]
    got = [[] for _ in range(nch)]
    want = [[] for _ in range(nch)]
    pos = 0
    for ln, g in ((12345, 0.8), (1, 0.8), (n - 12346, 0.8)):
        blk = torch.from_numpy(np.ascontiguousarray(bits[:, pos:pos + ln])).cuda()
        out = torch.empty((nch, max(ln, 1)), dtype=torch.float32, device="cuda")
        m = C.c_size_t()
        _lib.check(h, L.dsdgpu_decim_process(h, nch, C.c_void_p(blk.data_ptr()), blk.stride(0), ln,
                                             C.c_void_p(out.data_ptr()), out.stride(0), g, g,
                                             C.byref(m)))
        for c in range(nch):
            got[c].append(out[c, : m.value].cpu().numpy())
            y = refs[c].process(bits[c, pos:pos + ln].astype(np.float64) * 2 - 1)
            want[c].append((y * g).astype(np.float32))
        pos += ln
    for c in range(nch):
        a, b = np.concatenate(got[c]), np.concatenate(want[c])
        assert a.shape == b.shape
        np.testing.assert_allclose(a, b, rtol=0, atol=2e-7 * max(1e-30, np.abs(b).max()))
    L.dsdgpu_destroy(h)


def _sinad(y, fs, f0):
    n = len(y)
    lo, hi = n // 4, n - n // 20
    t = np.arange(lo, hi) / fs
    A = np.stack([np.sin(2 * np.pi * f0 * t), np.cos(2 * np.pi * f0 * t), np.ones_like(t)], 1)
    coef, *_ = np.linalg.lstsq(A, y[lo:hi].astype(np.float64), rcond=None)
    fit = A[:, :2] @ coef[:2]
    res = y[lo:hi] - A @ coef
    return 10 * np.log10(np.sum(fit * fit) / np.sum(res * res))


def test_dsd_to_pcm_pipeline_sinad(oracle):
    """PCM 997 Hz -> DSD128 (a plain sequential trellis encode on the GPU: the
    DAS seams would cap any SINAD near 56 dB) -> DoP -> the DSD -> PCM
    pipeline -> 44.1 kHz float: SINAD equal to the oracle chain's on the same
    DSD (within 0.01 dB) and above 115 dB."""
    from foo_dsd_trellis_gb300 import _lib, ntf, signals
    from foo_dsd_trellis_gb300.fir import FirChain
    from foo_dsd_trellis_gb300.pipeline import PCM_FIR_GAIN, Encoder
    from foo_dsd_trellis_gb300.sdm import TrellisSdm
    fs_pcm, fs_dsd, nch, K, depth, lat = 44100, 5644800, 2, 16, 32, 32
    f = ntf.get_filter("clans-7", fs_dsd)
    # no dither: the -110 dBFS TPDF of the small case would floor the SINAD
    pcm = signals.sine_tpdf(0.25, fs_pcm, nch, dither_db=-300.0, seed=9)
    g = float(PCM_FIR_GAIN)
    fir = FirChain(fs_pcm, fs_dsd, boxcar_taps=8, soft_clip=True, num_channels=nch).process(
        torch.from_numpy(pcm).cuda(), g, g)
    sdm = TrellisSdm(f.order, f.a, f.g, depth, K, lat, num_contexts=nch)
    body = sdm.process_block(fir)
    tail = sdm.drain(lat, nch=nch)
    dsd = np.stack([np.concatenate([body[c].cpu().numpy(), tail[c].cpu().numpy()]) for c in range(nch)])
    ns = dsd.shape[1] - dsd.shape[1] % 128
    dsd = dsd[:, :ns]
    dop = np.stack([oracle.dop_float_frames(dsd[c], 0) for c in range(nch)])
    dec = Encoder(fs_dsd, fs_pcm, nch, f, depth, K, lat, output_format=_lib.OUT_PCM)
    out = torch.empty((nch, ns // 128 + 16), dtype=torch.float32, device="cuda")
    n_out, nbytes = dec.process(torch.from_numpy(dop).cuda(), out, 1.0, 1.0)
    assert n_out == ns // 128 and nbytes == 4 * n_out * nch
    got = out[:, :n_out].cpu().numpy()
    for c in range(nch):
        ref = oracle.Decimator(fs_dsd, fs_pcm).process(dsd[c].astype(np.float64) * 2 - 1)
        ref = ref.astype(np.float32)          # the reference narrows to float too
        s_got, s_ref = _sinad(got[c], fs_pcm, 997.0), _sinad(ref, fs_pcm, 997.0)
        assert abs(s_got - s_ref) < 0.01, (s_got, s_ref)
        assert s_got > 115.0, s_got
