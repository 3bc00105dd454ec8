"""Host-side logic on CPU: FIR stage planning, tap design and the Python
mirrors' parameter checks, against the oracle."""
import numpy as np
import pytest


def test_fir_plan_matches_oracle(oracle):
    for fs_in in (44100, 48000, 88200, 96000, 176400, 192000, 2822400, 3072000, 5644800):
        for k in range(1, 10):
            fs_out = fs_in * (1 << k)
            plan = oracle.fir_plan(fs_in, fs_out)
            assert sum(1 for _ in plan) >= 1
            if fs_out in (22579200, 24576000) and k == 3:
                assert plan == [(4, 127), (2, 63)]
            elif fs_out in (22579200, 24576000) and k >= 2:
                assert plan[0] == (2, 127) and all(p == (2, 63) for p in plan[1:])
            else:
                assert all(p == (2, 63) for p in plan)


def test_halfband_design_properties(oracle):
    h = oracle.fir_design(63)
    assert abs(h.sum() - 1.0) < 1e-15
    assert np.array_equal(h, h[::-1])
    assert abs(h[31] - 0.5) < 1e-6
    assert np.all(np.abs(h[1::2][np.arange(31) != 15]) < 1e-15)   # half-band zeros
    q = oracle.fir_design(127, quarter=True)
    assert abs(q.sum() - 1.0) < 1e-15


def _goertzel_power(x, f, fs):
    w = 2 * np.pi * f / fs
    coeff = 2 * np.cos(w)
    s1 = s2 = 0.0
    for v in x:
        s0 = v + coeff * s1 - s2
        s2, s1 = s1, s0
    return (s1 * s1 + s2 * s2 - coeff * s1 * s2) / (len(x) * len(x))


def test_fir_chain_passband_and_images(oracle):
    """The reference's own FIR checks on DSD64 -> DSD128 (test/test_fir.c:168-257):
    passband flat within 0.1 dB to 20 kHz, the image at fs_in - f below -80 dB,
    output count = in * 2.  Tones sit on an FFT bin of the input block."""
    fs_in, fs_out, n_in = 2822400, 5644800, 16384
    for f0 in (1000.0, 5000.0, 10000.0, 15000.0, 20000.0):
        bin_in = fs_in / n_in
        fx = round(f0 / bin_in) * bin_in
        t = np.arange(n_in)
        x = (0.5 * np.sin(2 * np.pi * fx * t / fs_in)).astype(np.float32)
        y = oracle.engine_fir(fs_in, fs_out, x, boxcar_taps=0, soft_clip=False)
        assert len(y) == 2 * n_in
        p_in = _goertzel_power(x.astype(np.float64), fx, fs_in)
        p_out = _goertzel_power(y, fx, fs_out)
        assert abs(10 * np.log10(p_out / p_in)) < 0.1
        if f0 == 10000.0:
            p_img = _goertzel_power(y, fs_in - fx, fs_out)
            assert 10 * np.log10(p_img / p_out) < -80


def test_ntf_auto_latency_rules():
    from foo_dsd_trellis_gb300 import ntf
    assert ntf.auto_latency(44100, ntf.DSD_RATE_64) == 32
    assert ntf.auto_latency(48000, ntf.DSD48_RATE_128) == 128
    assert ntf.auto_latency(48000, ntf.DSD48_RATE_256) == 128
    assert ntf.auto_latency(48000, ntf.DSD48_RATE_512) == 32
    assert ntf.auto_select(ntf.DSD_RATE_64).name == "clans-5"
    assert ntf.auto_select(ntf.DSD_RATE_128).name == "clans-6"
    assert ntf.auto_select(ntf.DSD_RATE_512).name == "clans-8"


def test_das_oracle_structural_properties(oracle):
    """One segment equals the plain SDM; seg0-first with two segments (seg1
    DIRECT from seg0's end state) also equals the plain SDM."""
    from signals import multitone
    from foo_dsd_trellis_gb300 import ntf
    f = ntf.get_filter("clans-6", ntf.DSD_RATE_128)
    a, g = np.array(f.a), np.array(f.g)
    x = multitone(40000, 3) * 2.0
    plain = oracle.sdm_bits(oracle.sdm(f.order, a, g, 16, 8, 16), x)
    b1, _, _ = oracle.das_run(f.order, a, g, 16, 8, 16, 0.0, x, nsegs=1)
    b2, _, _ = oracle.das_run(f.order, a, g, 16, 8, 16, 0.0, x, nsegs=2, seed_mode=1)
    assert np.array_equal(b1[0], plain) and np.array_equal(b2[0], plain)
    b6, seams, starts = oracle.das_run(f.order, a, g, 16, 8, 16, 0.0, x, nsegs=6, seed_mode=0)
    # full-parallel: seg0 is cut back to its nominal length before the first overlap
    assert b6.shape[1] == len(x) - 64 * 16


def test_oracle_dsd_down_branch_streams(oracle):
    """The oracle's DSD -> DSD downsampling branch (boxcar, FP64 decimation,
    gain, clip) carries its state: two chunks equal one pass, and with unit
    gain and no clip it is the decimation of the boxcar mean."""
    import numpy as np
    rng = np.random.default_rng(4)
    x = np.where(rng.random(40000) > 0.5, 1.0, -1.0).astype(np.float32)
    one = oracle.engine_down(oracle.Boxcar(8), oracle.Decimator(5644800, 2822400), x, 0.7, 0.7, True)
    bc, dec = oracle.Boxcar(8), oracle.Decimator(5644800, 2822400)
    two = np.concatenate([oracle.engine_down(bc, dec, x[:12346], 0.7, 0.7, True),
                          oracle.engine_down(bc, dec, x[12346:], 0.7, 0.7, True)])
    assert np.array_equal(one, two)
    plain = oracle.engine_down(oracle.Boxcar(8), oracle.Decimator(11289600, 2822400), x, 1.0, 1.0, False)
    mean = oracle.Boxcar(8).process(x, 1.0, 1.0)
    assert np.array_equal(plain, oracle.Decimator(11289600, 2822400).process(mean))


def test_reference_citations_resolve():
    """Every reference file:line cited in the repository's tracked files
    exists in the reference tree (checked where the oracle is built)."""
    import pytest
    from oracle import check_citations
    if not check_citations.reference_present():
        pytest.skip("reference tree not present")
    bad = check_citations.bad_citations()
    assert not bad, bad[:10]


def _quant_fast(u: float, levels: int):
    """The estimator's quantiser shortcut, restated on the bits of u (as the
    CUDA step forms them): floor(u + 0.5) clamped to [0, levels - 1], or None
    where the reference's divisions must decide."""
    import struct
    b = struct.unpack("<Q", struct.pack("<d", u))[0]
    hi, lo = b >> 32, b & 0xFFFFFFFF
    ex = (hi >> 20) & 0x7FF
    sh = 1035 - min(max(ex, 1021), 1032)
    mh = (hi & 0xFFFFF) | 0x100000
    fl = (((mh << 32) | lo) >> sh) & 0xFFFFFFFF
    fh = mh >> sh
    f8 = fh & 0xFF
    near = (f8 == 0x80 and fl <= 1100) or (f8 == 0x7F and fl >= 2**32 - 1100)
    low = (hi >> 31) != 0 or ex < 1021
    if ex >= 1033 or (not low and near):
        return None
    return 0 if low else min((fh + 0x80) >> 8, levels - 1)


def test_estimator_quantiser_shortcut():
    """sdm_estimate_state_multibit's index trunc((v / a0 + 1) / step + 0.5)
    (src/trellis.c:1162-1166, FP64) equals the shortcut floor(u + 0.5) with
    u = fma(v, 1/(a0 step), 1/step) wherever the shortcut decides: random v,
    and v placed a few ulps and 1e-12 .. 2e-9 from every level boundary, for
    3, 16, 32 and 97 levels and four a0."""
    from fractions import Fraction as Fr
    rng = np.random.default_rng(7)
    for levels in (3, 16, 32, 97):
        step = 2.0 / (levels - 1)
        rstep = 1.0 / step
        for a0 in (0.51234, 1.7, 0.0923, 3.3e-3):
            c1 = (1.0 / a0) * rstep
            vs = list(rng.standard_normal(300) * a0 * 1.5)
            for k in range(levels + 1):
                v0 = ((k - 0.5) * step - 1.0) * a0
                sp = np.spacing(v0) if v0 != 0.0 else 5e-324
                vs += [v0 + d * sp for d in range(-4, 5)]
                for rel in (1e-12, 1e-9, 2e-9):
                    vs += [v0 * (1 + rel) + rel * a0, v0 * (1 - rel) - rel * a0]
            decided = 0
            for i, v in enumerate(vs):
                v = float(v)
                u = float(Fr(v) * Fr(c1) + Fr(rstep))          # one rounding: the fma
                q = _quant_fast(u, levels)
                w = (v / a0 + 1.0) / step + 0.5
                ref = max(0, min(int(w), levels - 1))
                if q is not None:
                    decided += i < 300
                    assert q == ref, (levels, a0, v)
            assert decided >= 290   # random inputs: the shortcut decides nearly all
