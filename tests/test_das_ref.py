"""Pins the oracle's Density-Aligned Stitching (oracle/das_oracle.c) to the
reference's own plugin_process (src/dsp_plugin.c:1146-2990), compiled here
with the reference's engine, FIR chain and trellis (oracle/ref_plugin.c; Win32
and Intel IPP replaced by stand-ins, the thread pool run inline).

The plugin converts interleaved DoP input: DoP unpack, the engine's FIR phase
(src/engine.c:790-900), DAS layout, reposition, seeding, segment SDM, seam
search, assembly, state carry (src/dsp_plugin.c:1343-2725) and DoP packing.
The checker hands the plugin's own FIR output of each chunk to the oracle's
DAS with the trellis parameters the engine resolved, DoP-packs its decisions
with the running marker phase and interleaves the channels as the plugin
does; the bytes must be identical.  Skipped where the reference tree (and so
oracle/_ref) is absent."""
import numpy as np
import pytest

DSD512 = 22579200


@pytest.fixture(scope="module")
def plug(oracle):
    if oracle.ref_plugin_lib() is None:
        pytest.skip("reference build (oracle/_ref) not present")
    return oracle


def _dsd_input(fs, seconds, nch, quiet=None):
    """DoP frames [frames, nch] of a second-order sigma-delta of two tones per
    channel; `quiet` = (start, end) fractions replaced by DSD silence (0x69)."""
    from foo_dsd_trellis_gb300.signals import dop_floats
    n = int(fs * seconds) // 16 * 16
    t = np.arange(n) / fs
    cols = []
    for c in range(nch):
        x = 0.4 * np.sin(2 * np.pi * (997.0 + 311.0 * c) * t) + 0.1 * np.sin(2 * np.pi * 5123.0 * t)
        bits = np.empty(n, np.uint8)
        i1 = i2 = y = 0.0
        for k, v in enumerate(x.tolist()):
            i1 += v - y
            i2 += i1 - y
            b = i2 >= 0.0
            y = 1.0 if b else -1.0
            bits[k] = b
        if quiet is not None:
            a, e = int(quiet[0] * n) // 8 * 8, int(quiet[1] * n) // 8 * 8
            bits[a:e] = np.tile(np.unpackbits(np.array([0x69], np.uint8)), (e - a) // 8)
        cols.append(dop_floats(bits))
    return np.stack(cols, axis=1)


def _run(O, fs_in, fs_out, nch, K, depth, lat, par, seconds, chunks=1, quiet=None, **kw):
    dop = _dsd_input(fs_in, seconds, nch, quiet)
    plug = O.RefPlugin(fs_in, fs_out, nch, K, depth, lat, par_mode=par, **kw)
    e = plug.engine()
    assert e["sdm_mode"] == 1                      # SDM_MODE_TRELLIS
    carry = [O.sdm(e["order"], e["a"], e["g"], e["depth"], e["cands"], e["lat"], e["state_limit"])
             for _ in range(nch)]
    per = dop.shape[0] // chunks
    phase = 0
    info = []
    for k in range(chunks):
        got = plug.process(dop[k * per:(k + 1) * per])
        fir = plug.fir()
        segs = plug.segments()
        bits, seams, starts = O.das_run(e["order"], e["a"], e["g"], e["depth"], e["cands"],
                                        e["lat"], e["state_limit"], fir, nsegs=segs,
                                        seed_mode=1 if fs_out < DSD512 else 0, reposition=True,
                                        carry=carry)
        packs = [O.dop_pack_bits(bits[c], phase) for c in range(nch)]
        phase = packs[0][1]
        want = np.stack([p[0].reshape(-1, 3) for p in packs], axis=1).reshape(-1)
        assert len(got) == len(want), (k, len(got), len(want))
        bad = np.nonzero(got != want)[0]
        assert bad.size == 0, f"chunk {k}: {bad.size} bytes differ, first {bad[:4]}"
        info.append(dict(segments=segs, seams=seams, starts=starts, fir_count=fir.shape[1],
                         out=bits.shape[1]))
    return info


@pytest.mark.parametrize("fs_in,fs_out,K,depth,lat,par,seconds", [
    (2822400, 11289600, 8, 16, 32, -1, 0.06),    # x4, seg0-first, automatic count (2)
    (5644800, 11289600, 16, 32, 64, 8, 0.05),    # x2, seg0-first, estimator for seg2+
    (2822400, DSD512, 8, 16, 32, -1, 0.03),      # x8 (4x + 2x stages), full-parallel, 4
    (11289600, 11289600, 8, 16, 32, 8, 0.03),    # same rate (boxcar), seg0-first
    (DSD512, DSD512, 4, 8, 16, 8, 0.02),         # same rate, full-parallel
    (3072000, 12288000, 32, 32, 128, 6, 0.06),   # 48k family, K = 32 (act[32] quirk)
    (11289600, 5644800, 8, 16, 32, 4, 0.05),     # DSD256 -> DSD128 decimation
], ids=["dsd64_256_auto", "dsd128_256_par8", "dsd64_512_auto", "same256_par8",
        "same512_par8", "dsd64_256_48k_k32", "dsd256_128_par4"])
def test_das_oracle_equals_reference_plugin(plug, fs_in, fs_out, K, depth, lat, par, seconds):
    info = _run(plug, fs_in, fs_out, 2, K, depth, lat, par, seconds)
    assert info[0]["segments"] > 1
    # boundaries with a seam search (seg0-first joins seg1 directly); not all at zero
    searched = info[0]["seams"][2 if fs_out < DSD512 else 1:]
    assert not searched or any(s > 0 for s in searched)


def test_das_same_rate_fir_lowpass(plug):
    """The engine's FIR mode on the same-rate path (fir_lowpass, src/fir.c:795-872)."""
    _run(plug, 11289600, 11289600, 2, 8, 16, 32, 4, 0.03, fir_mode=1)


@pytest.mark.parametrize("fs_out", [11289600, DSD512], ids=["seg0_first", "full_parallel"])
def test_das_stream_state_carry(plug, fs_out):
    """Three chunks in a row: the persistent context continues in seg0 and is
    replaced by the last segment's final state after every chunk
    (src/dsp_plugin.c:2714-2721); the DoP marker phase runs on."""
    info = _run(plug, 2822400, fs_out, 2, 8, 16, 32, 4, 0.09 if fs_out < DSD512 else 0.06,
                chunks=3)
    lat = 32
    # first chunk: the latency fill is lost once (seg0-first) or the full-parallel
    # seg0 cut drops one overlap; later chunks come out at the FIR count (seg0-first)
    if fs_out < DSD512:
        assert info[0]["out"] == info[0]["fir_count"] - lat
        assert all(i["out"] == i["fir_count"] for i in info[1:])
    else:
        assert all(i["out"] == i["fir_count"] - 64 * lat for i in info)


def test_das_quiet_boundary_reposition(plug):
    """DSD silence (0x69, as many ones as zeros in every byte) around the
    seg-3 boundary of a same-rate re-encode: the boxcar averages it to zero,
    the plugin's RMS search moves the boundary (src/dsp_plugin.c:1959-2024),
    and the oracle moves it the same way."""
    info = _run(plug, 5644800, 5644800, 2, 8, 16, 32, 6, 0.06, quiet=(0.46, 0.54))
    n = info[0]["fir_count"]
    nominal = [s * (n // 6) + min(s, n % 6) for s in range(6)]
    assert list(info[0]["starts"]) != nominal


@pytest.mark.parametrize("fs_in,fs_out,chunks", [
    (2822400, 11289600, 2),     # 2 half-band stages up
    (2822400, DSD512, 1),       # 4x quarter-band + 2x stages
    (3072000, 24576000, 1),     # 48k family, 127-tap first stage of a 3-stage chain
    (11289600, 5644800, 2),     # FP64 decimation
    (22579200, 2822400, 1),     # three /2 stages
], ids=["up4", "up8_512", "up8_512_48k", "down2", "down8"])
def test_fir_phase_equals_reference_engine(plug, fs_in, fs_out, chunks):
    """The FIR phase of the plugin's DAS path, engine_process_fir_gain
    (src/engine.c:789-900) with the reference's own fir.c (stage plan, tap
    design, FP64 chain with delay lines carried over chunks), against the
    oracle's FP64 restatement of the same chain on the +-1 input with the
    path gain and no boxcar or clip: bit for bit.  IPP's arithmetic is the
    published FIRMR semantics on both sides, so this pins the plan, the taps
    and the glue."""
    O = plug
    nch = 1
    dop = _dsd_input(fs_in, 0.02 if fs_out > fs_in else 0.03, nch)
    plug_ = O.RefPlugin(fs_in, fs_out, nch, 4, 8, 16, par_mode=4)
    e = plug_.engine()
    gain = float(np.float32(e["fir_gain"]))
    per = dop.shape[0] // chunks
    if fs_out > fs_in:
        hist = np.zeros(0, np.float32)
    else:
        dec = O.Decimator(fs_in, fs_out)
        bc = O.Boxcar(1)
    for k in range(chunks):
        plug_.process(dop[k * per:(k + 1) * per])
        got = plug_.fir()[0]
        x = O.dop_unpack(dop[k * per:(k + 1) * per, 0])
        if fs_out > fs_in:
            # the chain is LTI with zero initial delay lines: restate it on the
            # whole input so far and take this chunk's outputs
            hist = np.concatenate([hist, x])
            full = O.engine_fir(fs_in, fs_out, hist, boxcar_taps=0, g_start=gain, g_end=gain,
                                soft_clip=False)
            want = full[-len(x) * (fs_out // fs_in):]
        else:
            want = O.engine_down(bc, dec, x, gain, gain, False)
        assert len(got) == len(want), (k, len(got), len(want))
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), (
            k, np.max(np.abs(got - want)))


def test_sequential_path_equals_reference_engine(plug):
    """With one segment per channel (TRELLIS_PAR_SEQUENTIAL) the plugin runs
    engine_process_block per channel (src/engine.c:600-729: boxcar 8, FIR
    chain, gain ramp, tanh soft clip, sdm_process_block): its DoP output over
    two chunks equals the oracle's FIR glue (boxcar, chain, gain, clip) and
    its trellis, pinned to trellis.c, continued across the chunks."""
    O = plug
    fs_in, fs_out, nch, K, depth, lat = 2822400, 11289600, 2, 8, 16, 32
    dop = _dsd_input(fs_in, 0.04, nch)
    p = O.RefPlugin(fs_in, fs_out, nch, K, depth, lat, par_mode=0)
    e = p.engine()
    gain = float(np.float32(e["fir_gain"]))
    ctx = [O.sdm(e["order"], e["a"], e["g"], depth, K, lat, e["state_limit"]) for _ in range(nch)]
    per = dop.shape[0] // 2
    hist = [np.zeros(0, np.float32) for _ in range(nch)]
    phase = 0
    for k in range(2):
        got = p.process(dop[k * per:(k + 1) * per])
        assert p.segments() == 1
        bits = []
        for c in range(nch):
            x = O.dop_unpack(dop[k * per:(k + 1) * per, c])
            hist[c] = np.concatenate([hist[c], x])
            full = O.engine_fir(fs_in, fs_out, hist[c], boxcar_taps=8, g_start=gain, g_end=gain,
                                soft_clip=True)
            bits.append(O.sdm_bits(ctx[c], full[-len(x) * (fs_out // fs_in):]))
        n = min(len(b) for b in bits) // 16 * 16
        packs = [O.dop_pack_bits(b[:n], phase) for b in bits]
        phase = packs[0][1]
        want = np.stack([q[0].reshape(-1, 3) for q in packs], axis=1).reshape(-1)
        assert len(got) == len(want)
        assert np.array_equal(got, want), k
