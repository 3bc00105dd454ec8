"""Batched multi-stream plan vs the oracle, stream by stream.

Each stream of a batch must equal the single-stream path from fresh state:
the GPU FIR chain (checked against the FP64 oracle elsewhere) feeds the
oracle's DAS restatement (full-parallel seeding, RMS reposition), whose
decisions are packed by the oracle's DoP / native packers.  Streams mix input
rates of both families, DSD128 and DSD256 targets (CLANS-6 and CLANS-8, two
SDM parameter sets in one plan), uneven lengths, and one stream with a quiet
stretch over a DAS boundary (the host reposition path between the graphs).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GAIN = 0.354


def _noise(frames, ch, seed, level=0.25):
    """Band-limited Gaussian noise, float32 [ch, frames] (a seeded moving-average
    low-pass of white noise, scaled to `level` RMS)."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((ch, frames + 16))
    k = np.ones(4) / 4.0
    y = np.stack([np.convolve(w[c], k, mode="same")[8:8 + frames] for c in range(ch)])
    y *= level / max(1e-12, float(np.sqrt(np.mean(y * y))))
    return y.astype(np.float32)


def _specs(cands=8, depth=16, lat=16):
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.batch import StreamSpec
    rates = [(44100, 5644800, 2100), (48000, 12288000, 900), (88200, 5644800, 3000),
             (96000, 12288000, 1700), (176400, 11289600, 3300), (192000, 6144000, 5000)]
    specs = []
    for i, (fi, fo, frames) in enumerate(rates):
        f = ntf.auto_select(fo)
        specs.append(StreamSpec(fi, fo, 2 if i != 3 else 1, frames, f, cands=cands, depth=depth,
                                lat=lat, gain=GAIN, boxcar_taps=8 if i % 2 == 0 else 0,
                                soft_clip=bool(i % 3), reposition=True))
    return specs


def _inputs(specs):
    xs = []
    for i, s in enumerate(specs):
        x = _noise(s.frames, s.channels, 100 + i)
        if i == 0:
            # quiet stretch around the DAS boundary at FIR sample 3 * 32768
            c = 3 * 32768 // (s.fs_out // s.fs_in)
            x[:, c - 60:c + 60] *= 1e-4
        xs.append(x)
    return xs


def _oracle_stream(oracle, s, x, seg_len, fmt):
    """The single-stream path for one stream: GPU FIR from fresh state, then
    the oracle's DAS and packers."""
    from foo_dsd_trellis_gb300.batch import OUT_BITS, OUT_DOP
    from foo_dsd_trellis_gb300.fir import FirChain
    fc = FirChain(s.fs_in, s.fs_out, boxcar_taps=s.boxcar_taps, soft_clip=s.soft_clip,
                  num_channels=s.channels)
    fir = fc.process(torch.from_numpy(x).cuda(), GAIN, GAIN).cpu().numpy()
    fc.close()
    bits, seams, starts = oracle.das_run(s.ntf.order, np.array(s.ntf.a), np.array(s.ntf.g),
                                         s.depth, s.cands, s.lat, 0.0, fir, seg_len=seg_len,
                                         seed_mode=0, reposition=s.reposition)
    if fmt == OUT_BITS:
        return bits, starts
    if fmt == OUT_DOP:
        per = [oracle.dop_pack_bits(bits[c], 0)[0].reshape(-1, 3) for c in range(s.channels)]
        return np.stack(per, axis=1).reshape(-1), starts
    return np.stack([oracle.bits_pack(bits[c]) for c in range(s.channels)]), starts


@pytest.mark.parametrize("fmt", [1, 0, 2], ids=["dop", "bits", "native"])
def test_batch_equals_single_stream(oracle, fmt):
    from foo_dsd_trellis_gb300.batch import BatchPlan
    specs = _specs()
    xs = _inputs(specs)
    plan = BatchPlan(specs, seg_len=32768, output_format=fmt)
    info = plan.info()
    assert info["classes"] == 2 and info["seg_len"] == 32768
    plan.load([torch.from_numpy(x).cuda() for x in xs])
    plan.run()
    moved = False
    for i, s in enumerate(specs):
        want, starts = _oracle_stream(oracle, s, xs[i], 32768, fmt)
        got = plan.out_view(i).cpu().numpy()
        if fmt == 2:
            got = got[:, : want.shape[1]]
        assert got.shape == want.shape, (i, got.shape, want.shape)
        bad = np.nonzero(got != want)
        assert bad[0].size == 0, f"stream {i}: mismatch at {list(zip(*bad))[:5]}"
        if i == 0:
            moved = int(starts[3]) != 3 * (s.frames * (s.fs_out // s.fs_in) // len(starts))
    assert moved, "the quiet stretch did not move a boundary: the reposition path was not covered"
    plan.close()


def test_batch_k32_depth64_lat128(oracle):
    """The DSD128 trellis of the batched workload (K = 32, depth 64, lat 128)."""
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.batch import OUT_DOP, BatchPlan, StreamSpec
    specs = [StreamSpec(48000, 6144000, 2, 1700, ntf.auto_select(6144000), gain=GAIN),
             StreamSpec(44100, 11289600, 1, 900, ntf.auto_select(11289600), gain=GAIN)]
    xs = [_noise(s.frames, s.channels, 7 + i) for i, s in enumerate(specs)]
    plan = BatchPlan(specs, seg_len=32768, output_format=OUT_DOP)
    outs = plan.run_host(xs)
    for i, s in enumerate(specs):
        want, _ = _oracle_stream(oracle, s, xs[i], 32768, OUT_DOP)
        assert np.array_equal(outs[i], want), f"stream {i}"
    plan.close()


def test_batch_autotune_replay_and_host_path():
    """seg_len 0 picks a tuned length; graph replays are deterministic; the
    host-buffer run equals the device run; the plain form runs."""
    from foo_dsd_trellis_gb300.batch import OUT_DOP, BatchPlan
    specs = _specs()
    xs = _inputs(specs)
    plan = BatchPlan(specs, seg_len=0, output_format=OUT_DOP)
    info = plan.info()
    assert info["seg_len"] in (32768, 49152, 65536, 98304, 131072)
    assert info["blocks_per_sm"] in (8, 12, 16) and info["predicted_ms"] > 0
    plan.load([torch.from_numpy(x).cuda() for x in xs])
    plan.run()
    first = [plan.out_view(i).cpu().numpy().copy() for i in range(len(specs))]
    plan.run()
    for i in range(len(specs)):
        assert np.array_equal(plan.out_view(i).cpu().numpy(), first[i])
    outs = plan.run_host(xs)
    for i in range(len(specs)):
        assert np.array_equal(outs[i], first[i])
    t = plan.times_ms()
    assert t["sdm"] > 0 and t["total"] >= t["sdm"]
    smp, sec = plan.time_plain(2)
    assert smp > 0 and sec > 0
    plan.close()


def test_batch_rejects_bad_streams():
    from foo_dsd_trellis_gb300 import _lib, ntf
    from foo_dsd_trellis_gb300.batch import BatchPlan, StreamSpec
    f = ntf.auto_select(5644800)
    with pytest.raises(_lib.DsdGpuError) as e:
        BatchPlan([StreamSpec(44100, 5644801, 2, 1000, f)])
    assert e.value.code == _lib.ERR_ARG
    with pytest.raises(_lib.DsdGpuError) as e:
        BatchPlan([StreamSpec(44100, 5644800, 9, 1000, f)])
    assert e.value.code == _lib.ERR_ARG
    with pytest.raises(_lib.DsdGpuError) as e:
        BatchPlan([StreamSpec(44100, 5644800, 2, 100000, f)], seg_len=32768, max_device_bytes=1 << 20)
    assert e.value.code == _lib.ERR_TOO_LARGE
    # an unknown SDM mode, and a PreCorr stream with an NTF order out of range
    L = _lib.load()
    h = C.c_void_p()
    assert L.dsdgpu_create(0, C.byref(h)) == 0
    p = C.c_void_p()
    d = StreamSpec(44100, 5644800, 2, 1000, f).desc()
    d.sdm_mode = 7
    assert L.dsdgpu_plan_create(h, C.byref(d), 1, 32768, _lib.OUT_BITS, 0, C.byref(p)) == _lib.ERR_ARG
    d = StreamSpec(44100, 5644800, 2, 1000, f, precorr=True).desc()
    d.sdm.order = 11
    assert L.dsdgpu_plan_create(h, C.byref(d), 1, 32768, _lib.OUT_BITS, 0, C.byref(p)) == _lib.ERR_ARG
    L.dsdgpu_destroy(h)


def _precorr_want(oracle, s, x, fmt):
    """A PreCorr stream from fresh state: its FIR chain without the soft clip
    (the engine does not clip ahead of PreCorr), then the oracle's PreCorr per
    channel (pinned to src/precorr.c), packed as the plan packs."""
    from foo_dsd_trellis_gb300.batch import OUT_BITS
    from foo_dsd_trellis_gb300.fir import FirChain
    fc = FirChain(s.fs_in, s.fs_out, boxcar_taps=s.boxcar_taps, soft_clip=False,
                  num_channels=s.channels)
    fir = fc.process(torch.from_numpy(x).cuda(), GAIN, GAIN).cpu().numpy()
    fc.close()
    bits = np.stack([oracle.PreCorr(s.ntf.order, np.array(s.ntf.a), np.array(s.ntf.g),
                                    s.state_limit).process(fir[c]) for c in range(s.channels)])
    if fmt == OUT_BITS:
        return bits
    per = [oracle.dop_pack_bits(bits[c], 0)[0].reshape(-1, 3) for c in range(s.channels)]
    return np.stack(per, axis=1).reshape(-1)


@pytest.mark.parametrize("fmt", [0, 1], ids=["bits", "dop"])
def test_batch_precorr_streams(oracle, fmt):
    """PreCorr streams in a batch beside trellis streams: two PreCorr parameter
    sets (DSD64 without the limiter; DSD128 at 44.1 and 48 kHz with limit 12,
    sharing one table when their NTFs agree), uneven lengths, a mono stream.
    Each PreCorr stream equals its chain followed by the oracle's PreCorr from
    fresh state; each trellis stream still equals the single-stream path."""
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.batch import BatchPlan, StreamSpec
    specs = _specs()[:2]
    for (fi, fo, frames, lim, ch) in [(44100, 2822400, 3000, 0.0, 2), (48000, 6144000, 1500, 12.0, 2),
                                      (44100, 5644800, 2200, 12.0, 1)]:
        specs.append(StreamSpec(fi, fo, ch, frames, ntf.auto_select_precorr(fo), gain=GAIN,
                                boxcar_taps=8, soft_clip=True, state_limit=lim, precorr=True))
    xs = _inputs(specs)
    plan = BatchPlan(specs, seg_len=32768, output_format=fmt)
    assert plan.info()["classes"] == 2
    plan.load([torch.from_numpy(x).cuda() for x in xs])
    plan.run()
    for i, s in enumerate(specs):
        if s.precorr:
            want = _precorr_want(oracle, s, xs[i], fmt)
            assert plan.out_samples(i) == s.frames * (s.fs_out // s.fs_in)
        else:
            want, _ = _oracle_stream(oracle, s, xs[i], 32768, fmt)
        got = plan.out_view(i).cpu().numpy()
        assert got.shape == want.shape, (i, got.shape, want.shape)
        assert np.array_equal(got, want), f"stream {i}"
    plan.close()


def test_batch_precorr_only():
    """A plan of PreCorr streams alone (no trellis launch, no seams), run twice:
    the second run equals the first (every run starts from fresh state), and
    the host-buffer form equals the device form."""
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.batch import OUT_DOP, BatchPlan, StreamSpec
    specs = [StreamSpec(44100, 2822400, 2, 4000, ntf.auto_select_precorr(2822400), gain=GAIN,
                        precorr=True),
             StreamSpec(96000, 12288000, 2, 1000, ntf.auto_select_precorr(12288000), gain=GAIN,
                        state_limit=12.0, precorr=True)]
    xs = [_noise(s.frames, s.channels, 71 + i) for i, s in enumerate(specs)]
    plan = BatchPlan(specs, seg_len=0, output_format=OUT_DOP)
    assert plan.info()["classes"] == 0 and plan.info()["jobs"] == 0
    plan.load([torch.from_numpy(x).cuda() for x in xs])
    plan.run()
    first = [plan.out_view(i).cpu().numpy().copy() for i in range(len(specs))]
    plan.run()
    for i in range(len(specs)):
        assert np.array_equal(plan.out_view(i).cpu().numpy(), first[i])
    outs = plan.run_host(xs)
    for i in range(len(specs)):
        assert np.array_equal(outs[i], first[i])
    plan.close()


def test_batch_small_k_path_table_parameters(oracle):
    """The engine's path-table trellis (K = 2, depth 4) through the batched plan:
    every stream equals the single-stream path."""
    from foo_dsd_trellis_gb300.batch import OUT_BITS, BatchPlan
    specs = _specs(cands=2, depth=4, lat=16)[:4]
    xs = _inputs(specs)
    plan = BatchPlan(specs, seg_len=32768, output_format=OUT_BITS)
    plan.load([torch.from_numpy(x).cuda() for x in xs])
    plan.run()
    for i, s in enumerate(specs):
        want, _ = _oracle_stream(oracle, s, xs[i], 32768, OUT_BITS)
        got = plan.out_view(i).cpu().numpy()
        assert got.shape == want.shape and np.array_equal(got, want), f"stream {i}"
    plan.close()


def test_batch_long_latency_with_a_short_one(oracle):
    """A stream at lat 600 (overlap 38,400: the wide-ring SDM kernel and the
    seam search in HBM scratch) beside one at lat 16, in one plan."""
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.batch import OUT_BITS, BatchPlan, StreamSpec
    specs = [StreamSpec(44100, 5644800, 2, 2600, ntf.auto_select(5644800), cands=4, depth=8,
                        lat=600, gain=GAIN),
             StreamSpec(48000, 6144000, 1, 1500, ntf.auto_select(6144000), cands=8, depth=16,
                        lat=16, gain=GAIN)]
    xs = [_noise(s.frames, s.channels, 31 + i) for i, s in enumerate(specs)]
    plan = BatchPlan(specs, seg_len=65536, output_format=OUT_BITS)
    assert plan.info()["classes"] == 2
    plan.load([torch.from_numpy(x).cuda() for x in xs])
    plan.run()
    for i, s in enumerate(specs):
        want, _ = _oracle_stream(oracle, s, xs[i], 65536, OUT_BITS)
        got = plan.out_view(i).cpu().numpy()
        assert got.shape == want.shape and np.array_equal(got, want), f"stream {i}"
    plan.close()


def _dop_input(oracle, rate, frames, nch, seed):
    """DoP floats [nch, frames] of a DSD bitstream at `rate` (a quick trellis
    encode of a multitone, as the same-rate pipeline tests use)."""
    from signals import multitone

    from foo_dsd_trellis_gb300 import ntf
    f = ntf.get_filter("clans-5", rate)
    out = []
    for c in range(nch):
        ctx = oracle.sdm(f.order, np.array(f.a), np.array(f.g), 8, 4, 8)
        x = multitone(16 * frames + 8, 7 + seed + c) * 1.5
        out.append(oracle.dop_float_frames(oracle.sdm_bits(ctx, x)[: 16 * frames], 0))
    return np.stack(out).astype(np.float32)


@pytest.mark.parametrize("fmt", [1, 0], ids=["dop", "bits"])
def test_batch_dsd_input_streams(oracle, fmt):
    """DoP input in a batch, as the pipeline takes it: same-rate DSD64 (the
    engine's default 32-tap boxcar) and DSD128 (64 taps given), DSD64 -> DSD128
    through the FIR chain on the unpacked +-1 values, DSD128 -> DSD64 (boxcar 8,
    one FP64 half-band /2 stage, soft clip), DSD256 -> DSD64 (no boxcar, two
    stages) and same-rate DSD128 through the 127-tap FIR lowpass, beside a PCM
    stream.
    Each stream equals the single-stream pipeline on a fresh context with the
    same parameters (itself checked against the oracle's unpack, boxcar, FIR
    and DAS in test_dsd_gpu.py)."""
    from foo_dsd_trellis_gb300 import _lib, ntf
    from foo_dsd_trellis_gb300.batch import OUT_BITS, BatchPlan, StreamSpec
    from foo_dsd_trellis_gb300.pipeline import FULL_PARALLEL, Encoder
    pcm_spec = _specs()[0]
    dsd = [(2822400, 2822400, 2, 12000, 0, False, False), (5644800, 5644800, 1, 9000, 64, False, False),
           (2822400, 5644800, 2, 6000, 8, True, False), (5644800, 2822400, 2, 12000, 8, True, False),
           (11289600, 2822400, 1, 16000, 0, False, False), (5644800, 5644800, 2, 9000, 0, False, True)]
    specs = [pcm_spec]
    xs = [_inputs([pcm_spec])[0]]
    for k, (fi, fo, ch, frames, box, clip, lp) in enumerate(dsd):
        specs.append(StreamSpec(fi, fo, ch, frames, ntf.auto_select(fo), cands=8, depth=16, lat=16,
                                gain=0.9, boxcar_taps=box, soft_clip=clip, reposition=True,
                                lowpass=lp))
        xs.append(_dop_input(oracle, fi, frames, ch, 40 + k))
    plan = BatchPlan(specs, seg_len=32768, output_format=fmt)
    plan.load([torch.from_numpy(x).cuda() for x in xs])
    plan.run()
    for i, s in enumerate(specs):
        got = plan.out_view(i).cpu().numpy()
        if i == 0:
            want, _ = _oracle_stream(oracle, s, xs[0], 32768, fmt)
        else:
            enc = Encoder(s.fs_in, s.fs_out, s.channels, s.ntf, s.depth, s.cands, s.lat,
                          seg_len=32768, seed_mode=FULL_PARALLEL, reposition=True,
                          boxcar_taps=s.boxcar_taps, soft_clip=s.soft_clip, output_format=fmt,
                          samerate_filter=_lib.SAMERATE_LOWPASS if s.lowpass else _lib.SAMERATE_BOXCAR)
            n_out = 16 * s.frames * s.fs_out // s.fs_in
            if fmt == OUT_BITS:
                buf = torch.empty((s.channels, n_out + 256), dtype=torch.uint8, device="cuda")
            else:
                buf = torch.empty(enc.out_capacity(s.frames) + 64, dtype=torch.uint8, device="cuda")
            ns, nb = enc.process(torch.from_numpy(xs[i]).cuda(), buf, 0.9, 0.9)
            want = buf[:, :ns].cpu().numpy() if fmt == OUT_BITS else buf[:nb].cpu().numpy()
            enc.close()
            assert plan.out_samples(i) == ns
        assert got.shape == want.shape, (i, got.shape, want.shape)
        assert np.array_equal(got, want), f"stream {i}"
    plan.close()


@pytest.mark.parametrize("fmt", [0, 1], ids=["bits", "dop"])
def test_batch_precorr_dsd_input(oracle, fmt):
    """PreCorr on DoP input in a batch: same-rate DSD64 (default boxcar, and the
    FIR lowpass), DSD64 ->
    DSD128 (FIR chain, FP32 out), DSD128 -> DSD64 (decimation chain, FP32 out),
    limiter on and off, beside a PreCorr PCM stream.  Each equals the
    single-stream pipeline in PreCorr mode (which narrows its FP64 stage output
    ahead of the walk; checked against the oracle in test_dsd_gpu.py)."""
    from foo_dsd_trellis_gb300 import _lib, ntf
    from foo_dsd_trellis_gb300.batch import OUT_BITS, BatchPlan, StreamSpec
    from foo_dsd_trellis_gb300.pipeline import FULL_PARALLEL, Encoder
    cases = [(44100, 2822400, 2, 3000, 8, 12.0, False), (2822400, 2822400, 2, 8000, 0, 0.0, False),
             (2822400, 5644800, 1, 5000, 8, 12.0, False), (5644800, 2822400, 2, 10000, 8, 0.0, False),
             (2822400, 2822400, 1, 8000, 0, 12.0, True)]
    specs, xs = [], []
    for k, (fi, fo, ch, frames, box, lim, lp) in enumerate(cases):
        specs.append(StreamSpec(fi, fo, ch, frames, ntf.auto_select_precorr(fo), gain=0.8,
                                boxcar_taps=box, soft_clip=True, state_limit=lim, precorr=True,
                                lowpass=lp))
        xs.append(_noise(frames, ch, 90) if fi < 2822400 else _dop_input(oracle, fi, frames, ch, 60 + k))
    plan = BatchPlan(specs, seg_len=32768, output_format=fmt)
    plan.load([torch.from_numpy(x).cuda() for x in xs])
    plan.run()
    for i, s in enumerate(specs):
        enc = Encoder(s.fs_in, s.fs_out, s.channels, s.ntf, 16, 8, 16, state_limit=s.state_limit,
                      seg_len=32768, seed_mode=FULL_PARALLEL, boxcar_taps=s.boxcar_taps,
                      soft_clip=True, output_format=fmt, sdm_mode=_lib.SDM_PRECORR,
                      samerate_filter=_lib.SAMERATE_LOWPASS if s.lowpass else _lib.SAMERATE_BOXCAR)
        n_out = (16 if s.fs_in >= 2822400 else 1) * s.frames * s.fs_out // s.fs_in
        if fmt == OUT_BITS:
            buf = torch.empty((s.channels, n_out + 256), dtype=torch.uint8, device="cuda")
        else:
            buf = torch.empty(enc.out_capacity(s.frames) + 64, dtype=torch.uint8, device="cuda")
        ns, nb = enc.process(torch.from_numpy(xs[i]).cuda(), buf, 0.8, 0.8)
        want = buf[:, :ns].cpu().numpy() if fmt == OUT_BITS else buf[:nb].cpu().numpy()
        enc.close()
        got = plan.out_view(i).cpu().numpy()
        assert plan.out_samples(i) == ns == n_out
        assert got.shape == want.shape, (i, got.shape, want.shape)
        assert np.array_equal(got, want), f"stream {i}"
    plan.close()


def test_batch_tiny_streams_every_mode(oracle):
    """One-frame and few-frame streams in every mode of the plan (PCM trellis,
    PCM PreCorr, same-rate DSD by boxcar and by lowpass, DSD up, DSD down by
    one and two stages, PreCorr on DoP input): no error, and each equals the
    single-stream pipeline on a fresh context (decision bytes)."""
    from foo_dsd_trellis_gb300 import _lib, ntf
    from foo_dsd_trellis_gb300.batch import OUT_BITS, BatchPlan, StreamSpec
    from foo_dsd_trellis_gb300.pipeline import FULL_PARALLEL, Encoder
    cases = [(44100, 2822400, 1, 1, False, False), (48000, 6144000, 2, 3, True, False),
             (2822400, 2822400, 1, 1, False, False), (5644800, 5644800, 2, 2, False, True),
             (2822400, 5644800, 1, 1, False, False), (5644800, 2822400, 2, 1, False, False),
             (11289600, 2822400, 1, 3, False, False), (2822400, 2822400, 1, 2, True, False)]
    specs, xs = [], []
    for k, (fi, fo, ch, frames, pc, lp) in enumerate(cases):
        f = ntf.auto_select_precorr(fo) if pc else ntf.auto_select(fo)
        specs.append(StreamSpec(fi, fo, ch, frames, f, cands=8, depth=16, lat=16, gain=0.7,
                                boxcar_taps=0 if fi == fo else 8, precorr=pc, lowpass=lp))
        xs.append(_noise(frames, ch, 200 + k) if fi < 2822400
                  else _dop_input(oracle, fi, frames, ch, 300 + k))
    plan = BatchPlan(specs, seg_len=32768, output_format=OUT_BITS)
    plan.load([torch.from_numpy(x).cuda() for x in xs])
    plan.run()
    for i, s in enumerate(specs):
        enc = Encoder(s.fs_in, s.fs_out, s.channels, s.ntf, 16, 8, 16, seg_len=32768,
                      seed_mode=FULL_PARALLEL, boxcar_taps=s.boxcar_taps, soft_clip=True,
                      output_format=OUT_BITS,
                      sdm_mode=_lib.SDM_PRECORR if s.precorr else _lib.SDM_TRELLIS,
                      samerate_filter=_lib.SAMERATE_LOWPASS if s.lowpass else _lib.SAMERATE_BOXCAR)
        n_out = (16 if s.fs_in >= 2822400 else 1) * s.frames * s.fs_out // s.fs_in
        buf = torch.zeros((s.channels, n_out + 256), dtype=torch.uint8, device="cuda")
        ns, _ = enc.process(torch.from_numpy(xs[i]).cuda(), buf, 0.7, 0.7)
        enc.close()
        want = buf[:, :ns].cpu().numpy()
        got = plan.out_view(i).cpu().numpy()
        assert plan.out_samples(i) == ns, (i, plan.out_samples(i), ns)
        assert got.shape == want.shape and np.array_equal(got, want), f"stream {i}"
    plan.close()
