"""PreCorr greedy SDM on the GPU, bit-exact against the oracle's restatement
(which the CPU suite pins to the reference's src/precorr.c): the trained
correction table, streamed decisions with and without the state limiter,
reset, and the whole pipeline in PreCorr mode."""
import numpy as np
import pytest

from signals import multitone

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("name,rate", [("clans-6", 2822400), ("clans-7", 5644800),
                                       ("clans-8", 11289600), ("clans-5", 2822400)])
def test_precorr_table(oracle, name, rate):
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.precorr import PreCorr
    f = ntf.get_filter(name, rate)
    got = PreCorr(f.order, f.a, f.g).table()
    want = oracle.PreCorr(f.order, np.array(f.a), np.array(f.g)).table()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("limit", [0.0, 12.0, 1.5])
def test_precorr_streamed(oracle, limit):
    """Four channels of different content, fed in ragged chunks (1, 15, 16, 17
    samples and longer) so state, history and phase cross every kind of
    boundary; the limiter at 1.5 clamps often."""
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.precorr import PreCorr
    f = ntf.auto_select_precorr(5644800)
    nch, n = 4, 60000
    x = np.stack([(0.3 + 0.15 * c) * multitone(n, 11 + c) for c in range(nch)])
    gpu = PreCorr(f.order, f.a, f.g, limit, num_channels=nch)
    refs = [oracle.PreCorr(f.order, np.array(f.a), np.array(f.g), limit) for _ in range(nch)]
    d_x = torch.from_numpy(x).cuda()
    cuts = [0, 1, 16, 32, 49, 1049, 21000, n]
    for lo, hi in zip(cuts[:-1], cuts[1:]):
        got = gpu.process_block(d_x[:, lo:hi]).cpu().numpy()
        for c in range(nch):
            assert np.array_equal(got[c], refs[c].process(x[c, lo:hi])), (c, lo, hi)


def test_precorr_channel_range_and_reset(oracle):
    """A call on a channel sub-range touches only those states; reset returns
    every channel to the initial state with the table kept."""
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.precorr import PreCorr
    f = ntf.auto_select_precorr(2822400)
    x = np.stack([0.4 * multitone(5000, 21 + c) for c in range(3)])
    d_x = torch.from_numpy(x).cuda()
    gpu = PreCorr(f.order, f.a, f.g, num_channels=3)
    gpu.process_block(d_x[1:2], first=1)
    both = gpu.process_block(d_x[0:1], first=0).cpu().numpy()[0]
    assert np.array_equal(both, oracle.PreCorr(f.order, np.array(f.a), np.array(f.g)).process(x[0]))
    r1 = oracle.PreCorr(f.order, np.array(f.a), np.array(f.g))
    r1.process(x[1])
    assert np.array_equal(gpu.process_block(d_x[1:2], first=1).cpu().numpy()[0], r1.process(x[1]))
    gpu.reset()
    got = gpu.process_block(d_x).cpu().numpy()
    for c in range(3):
        assert np.array_equal(got[c], oracle.PreCorr(f.order, np.array(f.a), np.array(f.g)).process(x[c]))


def test_precorr_empty_and_single():
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.precorr import PreCorr
    f = ntf.auto_select_precorr(2822400)
    gpu = PreCorr(f.order, f.a, f.g, num_channels=2)
    assert gpu.process_block(torch.zeros((2, 0), dtype=torch.float64, device="cuda")).shape == (2, 0)
    one = gpu.process_block(torch.zeros((2, 1), dtype=torch.float64, device="cuda")).cpu().numpy()
    assert one.shape == (2, 1)


def test_pipeline_precorr_mode(oracle):
    """PCM -> FIR chain -> PreCorr -> decision bytes through the pipeline equals
    the FIR chain run on its own followed by the oracle's PreCorr."""
    from foo_dsd_trellis_gb300 import _lib, ntf, signals
    from foo_dsd_trellis_gb300.fir import FirChain
    from foo_dsd_trellis_gb300.pipeline import OUT_BITS, PCM_FIR_GAIN, Encoder
    fs_in, fs_out, nch = 44100, 5644800, 2
    f = ntf.auto_select_precorr(fs_out)
    pcm = signals.sine_tpdf(0.05, fs_in, nch, seed=3)
    gain = float(PCM_FIR_GAIN)
    enc = Encoder(fs_in, fs_out, nch, f, 32, 8, 32, state_limit=12.0, output_format=OUT_BITS,
                  sdm_mode=_lib.SDM_PRECORR)
    n_fir = pcm.shape[1] * (fs_out // fs_in)
    out = torch.empty((nch, n_fir + 256), dtype=torch.uint8, device="cuda")
    ns, _ = enc.process(torch.from_numpy(pcm).cuda(), out, gain, gain)
    assert ns == n_fir
    got = out[:, :ns].cpu().numpy()
    # the engine does not soft-clip ahead of PreCorr (src/engine.c:704-717):
    # the pipeline drops the clip it was given
    fc = FirChain(fs_in, fs_out, boxcar_taps=8, soft_clip=False, num_channels=nch)
    fir = fc.process(torch.from_numpy(pcm).cuda(), gain, gain).cpu().numpy()
    for c in range(nch):
        y = fir[c]
        want = oracle.PreCorr(f.order, np.array(f.a), np.array(f.g), 12.0).process(y)
        assert np.array_equal(got[c], want), c


@pytest.mark.parametrize("order", [2, 3, 4, 9, 10])
def test_precorr_orders(oracle, order):
    """PreCorr at orders outside the NTF table (a real NTF truncated to order
    2, 3 or zero-padded to 9, 10, which keeps the loop bounded): table and
    decisions equal the restatement."""
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.precorr import PreCorr
    f = ntf.get_filter("clans-4", 2822400) if order <= 4 else ntf.get_filter("clans-8", 11289600)
    a, g = np.zeros(order), np.zeros(order)
    m = min(order, f.order)
    a[:m], g[:m] = np.array(f.a[:m]), np.array(f.g[:m])
    gpu = PreCorr(order, a, g, 5.0, num_channels=2)
    ref = [oracle.PreCorr(order, a, g, 5.0) for _ in range(2)]
    assert np.array_equal(gpu.table().view(np.uint32), ref[0].table().view(np.uint32))
    x = np.stack([0.4 * multitone(20000, 50 + order), 0.3 * multitone(20000, 60 + order)])
    got = gpu.process_block(torch.from_numpy(x).cuda()).cpu().numpy()
    for c in range(2):
        assert np.array_equal(got[c], ref[c].process(x[c]))
