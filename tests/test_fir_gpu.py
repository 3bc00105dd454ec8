"""GPU FIR chain (FP32 polyphase + FP64 glue) vs the FP64 oracle.

Tolerance: max |y_gpu - y_oracle| <= 1e-6 * max |y_oracle| over the block
(FIR output within 1e-6 relative of an FP64 oracle).  The oracle states the
reference's FIRMR semantics in direct form; the reference's own IPP result is
not available, so this pins the chain to the published algorithm."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1e-6


def _pcm(n, seed, amp=0.5):
    rng = np.random.Generator(np.random.PCG64(seed))
    t = np.arange(n)
    x = amp * np.sin(2 * np.pi * 997.0 / 44100.0 * t) + 0.05 * (rng.random(n) - rng.random(n))
    return x.astype(np.float32)


RATES = [
    (88200, 2822400),      # 5 stages to DSD64 (the whole-chain kernel's smallest factor)
    (44100, 2822400),      # 6 stages to DSD64
    (48000, 6144000),      # 7 stages to DSD128/48
    (44100, 11289600),     # 8 stages to DSD256 (the whole-chain kernel's largest factor)
    (88200, 11289600),     # 7 stages to DSD256
    (192000, 24576000),    # 7 stages, 127-tap first stage (to DSD512/48)
    (2822400, 22579200),   # ratio 8 to DSD512: 4x quarter-band + 2x
    (44100, 22579200),     # 9 stages
    (2822400, 5644800),    # 1 stage
]


@pytest.mark.parametrize("rates", RATES, ids=[f"{a}-{b}" for a, b in RATES])
def test_fir_chain_vs_fp64_oracle(oracle, rates):
    from foo_dsd_trellis_gb300.fir import FirChain
    fs_in, fs_out = rates
    ratio = fs_out // fs_in
    n = max(64, 60000 // ratio)
    x = _pcm(n, seed=ratio)
    want = oracle.engine_fir(fs_in, fs_out, x, boxcar_taps=8, g_start=0.354, g_end=0.354,
                             soft_clip=True)
    fc = FirChain(fs_in, fs_out, boxcar_taps=8, soft_clip=True)
    got = fc.process(torch.from_numpy(x).cuda(), 0.354, 0.354)[0].cpu().numpy()
    assert got.shape == want.shape
    err = np.abs(got - want).max() / np.abs(want).max()
    assert err <= TOL, f"relative error {err:.3g}"


def test_fir_streaming_blocks_equal_one_block(oracle):
    """Blocks with carried history equal one long block (delay-line continuity)."""
    from foo_dsd_trellis_gb300.fir import FirChain
    x = _pcm(5000, seed=9)
    want = oracle.engine_fir(48000, 6144000, x, boxcar_taps=8, soft_clip=True)
    fc = FirChain(48000, 6144000, boxcar_taps=8, soft_clip=True)
    parts, pos = [], 0
    for b in [1, 7, 100, 1000, 1, 2891, 1000]:
        parts.append(fc.process(torch.from_numpy(x[pos:pos + b].copy()).cuda())[0].cpu().numpy())
        pos += b
    got = np.concatenate(parts)
    assert pos == len(x)
    err = np.abs(got - want).max() / np.abs(want).max()
    assert err <= TOL, f"relative error {err:.3g}"


def test_fir_gain_ramp_and_das_phase(oracle):
    """DAS FIR phase: no boxcar, no clip, a gain ramp across the block."""
    from foo_dsd_trellis_gb300.fir import FirChain
    x = _pcm(4000, seed=4, amp=0.9)
    want = oracle.engine_fir(44100, 5644800, x, boxcar_taps=0, g_start=0.5, g_end=0.708,
                             soft_clip=False)
    fc = FirChain(44100, 5644800, boxcar_taps=0, soft_clip=False)
    got = fc.process(torch.from_numpy(x).cuda(), 0.5, 0.708)[0].cpu().numpy()
    err = np.abs(got - want).max() / np.abs(want).max()
    assert err <= TOL, f"relative error {err:.3g}"


def test_fir_multichannel(oracle):
    from foo_dsd_trellis_gb300.fir import FirChain
    xs = np.stack([_pcm(3000, seed=s) for s in range(4)])
    fc = FirChain(44100, 2822400, num_channels=4)
    got = fc.process(torch.from_numpy(xs).cuda()).cpu().numpy()
    for c in range(4):
        want = oracle.engine_fir(44100, 2822400, xs[c], boxcar_taps=8, soft_clip=True)
        err = np.abs(got[c] - want).max() / np.abs(want).max()
        assert err <= TOL


def test_integer_pipe_widening_equals_hardware():
    """The chain's epilogue widens every FP32 output to FP64 on the integer
    pipe: every one of the 2^32 binary32 patterns gives the hardware
    conversion's bits (NaNs as NaN)."""
    import ctypes as C
    from foo_dsd_trellis_gb300 import _lib
    L = _lib.load()
    h = C.c_void_p()
    assert L.dsdgpu_create(0, C.byref(h)) == _lib.OK
    bad = C.c_uint64(123)
    _lib.check(h, L.dsdgpu_selftest_convert(h, 1 << 32, 0, C.byref(bad)))
    assert bad.value == 0
    L.dsdgpu_destroy(h)
