"""UPOLS convolution vs exact FP64 linear convolution (the reference's
overlap-save convolver computes y[n] = sum_k h[k] x[n - k] with zero history,
src/convolution.c:355-405).  The GPU runs in FP32 (cuFFT transforms, the
partitioned multiply-accumulate kernel): max |y_gpu - y| <= 2e-5 * max |y|."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 2e-5


def _exact(x: np.ndarray, h: np.ndarray) -> np.ndarray:
    n = x.shape[-1]
    m = 1 << int(np.ceil(np.log2(n + h.shape[-1])))
    return np.fft.irfft(np.fft.rfft(x, m) * np.fft.rfft(h, m), m)[..., :n]


def _ir(nch, taps, seed):
    rng = np.random.default_rng(seed)
    h = rng.standard_normal((nch, taps)) * np.exp(-np.arange(taps) / (taps / 3.0))
    return (h / np.abs(h).max(axis=1, keepdims=True) * 0.05).astype(np.float32)


@pytest.mark.parametrize("taps,partition", [(65536, 4096), (1000, 256), (4096, 4096), (300, 64)])
def test_conv_matches_exact(taps, partition):
    from foo_dsd_trellis_gb300.conv import Convolver
    nch, n = 3, 200000 + 17
    rng = np.random.default_rng(taps)
    x = rng.standard_normal((nch, n)) * 0.3
    h = _ir(nch, taps, 1)
    cv = Convolver(h, partition)
    got = cv.process(torch.from_numpy(x).cuda()).cpu().numpy()
    want = _exact(x, h.astype(np.float64))
    err = np.abs(got - want).max()
    assert err <= TOL * np.abs(want).max(), (err, np.abs(want).max())
    cv.close()


def test_conv_streaming_history():
    """Uneven chunks with the history carried equal one pass."""
    from foo_dsd_trellis_gb300.conv import Convolver
    nch, n = 2, 150000
    rng = np.random.default_rng(3)
    x = rng.standard_normal((nch, n)) * 0.3
    h = _ir(nch, 20000, 2)
    cv = Convolver(h, 2048)
    parts, pos = [], 0
    for ln in (1, 4095, 70000, 30001, n - 104097):
        parts.append(cv.process(torch.from_numpy(np.ascontiguousarray(x[:, pos:pos + ln])).cuda()).cpu().numpy())
        pos += ln
    got = np.concatenate(parts, axis=1)
    want = _exact(x, h.astype(np.float64))
    assert np.abs(got - want).max() <= TOL * np.abs(want).max()
    cv.reset()
    again = cv.process(torch.from_numpy(x).cuda()).cpu().numpy()
    assert np.abs(again - want).max() <= TOL * np.abs(want).max()


def test_pipeline_applies_conv():
    """The pipeline with an IR set equals FIR chain -> convolution -> DAS run
    stage by stage (the same kernels, bit for bit)."""
    from foo_dsd_trellis_gb300 import ntf, signals
    from foo_dsd_trellis_gb300.conv import Convolver
    from foo_dsd_trellis_gb300.das import DasChannels
    from foo_dsd_trellis_gb300.fir import FirChain
    from foo_dsd_trellis_gb300.pipeline import FULL_PARALLEL, OUT_BITS, PCM_FIR_GAIN, Encoder
    fs_in, fs_out, K, depth, lat, nch = 48000, 24576000, 16, 48, 32, 2
    f = ntf.auto_select(fs_out)
    pcm = signals.sine_tpdf(0.05, fs_in, nch, seed=5)
    h = _ir(nch, 65536, 9)
    gain = float(PCM_FIR_GAIN)
    enc = Encoder(fs_in, fs_out, nch, f, depth, K, lat, seg_len=262144, seed_mode=FULL_PARALLEL,
                  boxcar_taps=8, soft_clip=True, output_format=OUT_BITS)
    enc.set_conv(h, 4096)
    n_fir = pcm.shape[1] * (fs_out // fs_in)
    out = torch.empty((nch, n_fir + 256), dtype=torch.uint8, device="cuda")
    ns, _ = enc.process(torch.from_numpy(pcm).cuda(), out, gain, gain)
    fc = FirChain(fs_in, fs_out, boxcar_taps=8, soft_clip=True, num_channels=nch)
    fir = fc.process(torch.from_numpy(pcm).cuda(), gain, gain)
    y = Convolver(h, 4096).process(fir)
    d = DasChannels(f.order, f.a, f.g, depth, K, lat, num_channels=nch)
    want, _ = d.process_chunk(y, seg_len=262144, seed_mode=FULL_PARALLEL)
    assert ns == want.shape[1]
    assert torch.equal(out[:, :ns], want)
