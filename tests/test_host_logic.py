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
