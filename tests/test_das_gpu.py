"""GPU Density-Aligned Stitching vs the oracle's restatement: the stitched
decision streams and the chosen seams must be identical (bit-exact), for both
seeding modes, several channels, and a quiet boundary that triggers the RMS
reposition."""
import numpy as np
import pytest

from signals import multitone, uniform_noise

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _run(oracle, f, depth, K, lat, fir, **kw):
    from foo_dsd_trellis_gb300.das import DasChannels
    want, wseams, _ = oracle.das_run(f.order, np.array(f.a), np.array(f.g), depth, K, lat, 0.0,
                                     fir, **kw)
    d = DasChannels(f.order, f.a, f.g, depth, K, lat, num_channels=fir.shape[0])
    got, seams = d.process_chunk(torch.from_numpy(np.ascontiguousarray(fir)).cuda(), **kw)
    got = got.cpu().numpy()
    return want, wseams, got, seams


def _ntf(name, rate):
    from foo_dsd_trellis_gb300 import ntf
    return ntf.get_filter(name, rate)


@pytest.mark.parametrize("mode", [0, 1], ids=["full_parallel", "seg0_first"])
def test_das_small(oracle, mode):
    f = _ntf("clans-6", 5644800)
    x = np.stack([multitone(80000, 3) * 2.0, multitone(80000, 4) * 1.5])
    want, ws, got, gs = _run(oracle, f, 16, 8, 16, x, nsegs=7, seed_mode=mode)
    assert got.shape == want.shape
    assert list(gs) == list(ws)
    bad = np.nonzero(got != want)
    assert bad[0].size == 0, f"mismatch at {list(zip(*bad))[:5]}"


def test_das_k32_depth64_lat128(oracle):
    """The DSD128 configuration's trellis (K=32, depth 64, lat 128), overlap
    8192, 32768-sample nominal segments."""
    f = _ntf("clans-7", 6144000)
    x = np.stack([multitone(32768 * 6 + 1234, 8), multitone(32768 * 6 + 1234, 9)])
    want, ws, got, gs = _run(oracle, f, 64, 32, 128, x, seg_len=32768, seed_mode=0)
    assert got.shape == want.shape
    assert list(gs) == list(ws)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("mode", [0, 1], ids=["full_parallel", "seg0_first"])
def test_das_long_latency(oracle, mode):
    """lat 300 (overlap 64 * lat = 19,200) on the wide-ring kernel, both
    seeding modes."""
    f = _ntf("clans-6", 5644800)
    x = np.stack([multitone(200000, 21) * 1.8, multitone(200000, 22) * 1.4])
    want, ws, got, gs = _run(oracle, f, 16, 8, 300, x, seg_len=40000, seed_mode=mode)
    assert got.shape == want.shape
    assert list(gs) == list(ws)
    assert np.array_equal(got, want)


def test_das_quiet_boundary_reposition(oracle):
    """A near-silent stretch around a seg>=2 boundary moves it (RMS search)."""
    f = _ntf("clans-5", 2822400)
    n = 120000
    x = multitone(n, 12) * 2.0
    x[55000:65000] = uniform_noise(10000, 5, 1e-4)    # quiet around the boundary at 60000
    want, ws, got, gs = _run(oracle, f, 16, 4, 16, x[None, :], nsegs=6, seed_mode=1)
    assert list(gs) == list(ws)
    assert np.array_equal(got, want)


def test_das_several_quiet_boundaries(oracle):
    """Four neighbouring boundaries inside one near-silent stretch: all their
    candidate windows are evaluated in one RMS launch, and each move sees the
    neighbour constraints of the moves made before it, as in the reference's
    boundary-by-boundary scan."""
    f = _ntf("clans-5", 2822400)
    n = 160000
    x = multitone(n, 13) * 2.0
    x[35000:105000] = uniform_noise(70000, 6, 1e-4)   # boundaries at 40k, 60k, 80k, 100k
    want, ws, got, gs = _run(oracle, f, 16, 4, 16, x[None, :], nsegs=8, seed_mode=1)
    _, _, starts = oracle.das_run(f.order, np.array(f.a), np.array(f.g), 16, 4, 16, 0.0,
                                  x[None, :], nsegs=8, seed_mode=1)
    nominal = [s * (n // 8) for s in range(8)]
    assert sum(a != b for a, b in zip(starts, nominal)) >= 3
    assert list(gs) == list(ws)
    assert np.array_equal(got, want)


def test_das_single_segment_is_plain_sdm(oracle):
    f = _ntf("clans-6", 5644800)
    x = multitone(30000, 21)[None, :]
    want, ws, got, gs = _run(oracle, f, 32, 16, 32, x, nsegs=1, seed_mode=0)
    ref = oracle.sdm(f.order, np.array(f.a), np.array(f.g), 32, 16, 32)
    plain = oracle.sdm_bits(ref, x[0])
    assert np.array_equal(got[0], plain)
    assert np.array_equal(want[0], plain)


@pytest.mark.parametrize("K,depth", [(2, 4), (4, 8), (5, 8), (12, 16)])
def test_lanes_per_job_do_not_change_results(oracle, K, depth):
    """Every width of the job packing (2 .. 32 lanes, 16 .. 1 jobs per warp,
    and the automatic choice) gives the oracle's DAS output: small K with a
    short path mask takes the serial selection often, in different jobs of
    the same warp."""
    from foo_dsd_trellis_gb300 import _lib
    from foo_dsd_trellis_gb300.das import DasChannels
    import ctypes as C
    f = _ntf("clans-6", 5644800)
    x = np.stack([multitone(150000, 7) * 1.2, multitone(150000, 8) * 0.9, multitone(150000, 9)])
    want, ws, _ = oracle.das_run(f.order, np.array(f.a), np.array(f.g), depth, K, 16, 0.0, x,
                                 seg_len=8192, seed_mode=0)
    for lanes in (0, 2, 4, 8, 16, 32):
        if lanes and lanes < K:
            continue
        d = DasChannels(f.order, f.a, f.g, depth, K, 16, num_channels=3)
        _lib.check(d.h, d.L.dsdgpu_set_option(d.h, _lib.OPT_SDM_LANES, lanes))
        got, seams = d.process_chunk(torch.from_numpy(x).cuda(), seg_len=8192, seed_mode=0)
        assert list(seams) == list(ws), lanes
        assert np.array_equal(got.cpu().numpy(), want), lanes
        d.close()


def test_lanes_option_rejects_bad_widths():
    from foo_dsd_trellis_gb300 import _lib
    from foo_dsd_trellis_gb300.das import DasChannels
    f = _ntf("clans-6", 5644800)
    d = DasChannels(f.order, f.a, f.g, 8, 4, 16, num_channels=1)
    for bad in (1, 3, 12, 64, -2):
        assert d.L.dsdgpu_set_option(d.h, _lib.OPT_SDM_LANES, bad) == _lib.ERR_ARG


def test_balanced_launch_equals_plain():
    """Enough DAS segments to land 5 % above one warp per FP64 pipe: the
    SDM launch cuts the segments into 1,024-sample parts queued over one warp
    per pipe (DSDGPU_OPT_SDM_BALANCE); the stitched output and seams equal
    the plain one-segment-per-warp launch, which the other tests pin to the
    oracle, and the part boundaries are the streamed-block boundaries the
    oracle tests cover."""
    from foo_dsd_trellis_gb300 import _lib
    from foo_dsd_trellis_gb300.das import DasChannels
    f = _ntf("clans-7", 6144000)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    pipes = 4 * sms
    S = (pipes + pipes // 20) // 2 + 1            # segments per channel, 2 channels
    seg = 20000
    x = np.stack([multitone(S * seg, 30) * 1.6, multitone(S * seg, 31) * 1.3])
    fir = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    outs, kernels = [], []
    for balance in (1, 0):
        d = DasChannels(f.order, f.a, f.g, 16, 32, 32, num_channels=2)
        _lib.check(d.h, d.L.dsdgpu_set_option(d.h, _lib.OPT_SDM_BALANCE, balance))
        got, seams = d.process_chunk(fir, nsegs=S, seed_mode=0)
        outs.append((got.cpu().numpy(), list(seams)))
        kernels.append(d.last_sdm_kernel())
        d.close()
    assert kernels == ["sdm_parts_kernel<7>", "sdm_jobs_kernel<7,32>"]
    assert outs[0][1] == outs[1][1]
    assert np.array_equal(outs[0][0], outs[1][0])


def test_das_output_counts_over_chunks(oracle):
    """The plugin's DAS output check (src/dsp_plugin.c:2729-2745): in seg0-first
    mode a channel's first chunk comes out trellis_lat samples short of its
    FIR count (the latency fill) and every later chunk exactly at it, so
    chunks of a multiple of 16 keep the DoP frame alignment."""
    from foo_dsd_trellis_gb300.das import DasChannels
    f = _ntf("clans-6", 5644800)
    lat = 64
    d = DasChannels(f.order, f.a, f.g, 16, 8, lat, num_channels=2)
    for k, n in enumerate((160000, 96000, 131072)):
        x = np.stack([multitone(n, 40 + k) * 1.4, multitone(n, 50 + k) * 1.2])
        got, _ = d.process_chunk(torch.from_numpy(x).cuda(), seg_len=32768, seed_mode=1)
        want = n - lat if k == 0 else n
        assert got.shape == (2, want)
        assert want % 16 == 0
    d.close()


def test_pipeline_flush_restarts_the_stream():
    """dsdgpu_pipeline_flush (plugin_flush, src/dsp_plugin.c:3622-3653): a chunk
    after a flush equals the same chunk on a fresh pipeline, and differs from
    the chunk that continues the stream."""
    from foo_dsd_trellis_gb300 import ntf, signals
    from foo_dsd_trellis_gb300.pipeline import FULL_PARALLEL, OUT_DOP, Encoder
    f = ntf.get_filter("clans-7", 6144000)
    pcm = torch.from_numpy(signals.dsd128_multitone_pink(0.3, 48000, 2, 7)).cuda()

    def enc():
        return Encoder(48000, 6144000, 2, f, 32, 16, 64, seg_len=65536, seed_mode=FULL_PARALLEL,
                       output_format=OUT_DOP)
    a, b = enc(), enc()
    cap = a.out_capacity(pcm.shape[1]) + 64
    outs = []
    for e, flush in ((a, False), (b, True)):
        o1 = torch.zeros(cap, dtype=torch.uint8, device="cuda")
        o2 = torch.zeros(cap, dtype=torch.uint8, device="cuda")
        _, n1 = e.process(pcm, o1)
        if flush:
            e.flush()
        _, n2 = e.process(pcm, o2)
        outs.append((o1[:n1].cpu().numpy(), o2[:n2].cpu().numpy()))
    assert np.array_equal(outs[1][1], outs[0][0])          # flushed == fresh
    assert not np.array_equal(outs[0][1], outs[0][0])      # continued != fresh


@pytest.mark.parametrize("mode", [0, 1], ids=["full_parallel", "seg0_first"])
def test_das_stream_of_chunks_equals_oracle(oracle, mode):
    """Three chunks of one stream: the GPU's persistent contexts carry from
    chunk to chunk (seg0 continues them; the last segment's final state
    replaces them, src/dsp_plugin.c:2714-2721) exactly as the oracle's, which
    is pinned to the reference's plugin_process over chunk streams."""
    from foo_dsd_trellis_gb300.das import DasChannels
    f = _ntf("clans-6", 5644800)
    K, depth, lat = 8, 16, 32
    n = 3 * 90000
    x = np.stack([multitone(n, 51) * 1.7, multitone(n, 52) * 1.2])
    carry = [oracle.sdm(f.order, np.array(f.a), np.array(f.g), depth, K, lat) for _ in range(2)]
    d = DasChannels(f.order, f.a, f.g, depth, K, lat, num_channels=2)
    for k in range(3):
        chunk = np.ascontiguousarray(x[:, k * 90000:(k + 1) * 90000])
        want, ws, _ = oracle.das_run(f.order, np.array(f.a), np.array(f.g), depth, K, lat, 0.0,
                                     chunk, nsegs=5, seed_mode=mode, carry=carry)
        got, gs = d.process_chunk(torch.from_numpy(chunk).cuda(), nsegs=5, seed_mode=mode)
        assert list(gs) == list(ws), k
        assert np.array_equal(got.cpu().numpy(), want), k
    d.close()
