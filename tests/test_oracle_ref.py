"""Pins the oracle: the C restatement (oracle/sdm_oracle.c, pack_oracle.c) must
equal the reference's own trellis.c / dop.c, compiled from the reference sources
into oracle/_ref/.  Skipped where the reference tree (and so oracle/_ref) is
absent."""
import ctypes as C

import numpy as np
import pytest

from signals import multitone, sdm_input


@pytest.fixture(scope="module")
def ref(oracle):
    r = oracle.ref_lib()
    if r is None:
        pytest.skip("reference build (oracle/_ref) not present")
    return r


@pytest.fixture(scope="module")
def wide(oracle):
    r = oracle.ref_lib(True)
    if r is None:
        pytest.skip("reference build (oracle/_ref) not present")
    return r


def _table(ref, oracle):
    L = ref.lib
    a = np.zeros(10)
    g = np.zeros(10)
    order = C.c_int()
    freq = C.c_uint()
    name = C.create_string_buffer(64)
    out = []
    for i in range(L.ref_ntf_count()):
        L.ref_ntf_entry(i, a.ctypes.data_as(oracle._dp), g.ctypes.data_as(oracle._dp),
                        C.byref(order), C.byref(freq), name, 64)
        out.append((name.value.decode(), order.value, freq.value, a.copy(), g.copy()))
    return out


def test_ntf_table_bit_identical(ref, oracle):
    from foo_dsd_trellis_gb300 import ntf
    t = _table(ref, oracle)
    assert len(t) == len(ntf.TABLE)
    for (nm, order, freq, a, g), e in zip(t, ntf.TABLE):
        assert (nm, order, freq) == (e.name, e.order, e.freq)
        assert np.array_equal(a[:order], np.array(e.a)) and np.array_equal(g[:order], np.array(e.g))


def test_ntf_lookup_rules(ref, oracle):
    from foo_dsd_trellis_gb300 import ntf
    rates = [2822400, 3072000, 5644800, 6144000, 11289600, 12288000, 22579200, 24576000,
             45158400, 90316800, 1000]
    for rate in rates:
        for i in range(10):
            idx = ref.lib.ref_ntf_lookup(i, rate)
            if idx < 0:
                with pytest.raises(KeyError):
                    ntf.get_filter(i, rate)
            else:
                assert ntf.get_filter(i, rate).index == idx
        ai = ref.lib.ref_ntf_auto(rate)
        if ai >= 0:
            assert ntf.auto_select(rate).index == ai


def _cmp(oracle, lib, f, depth, K, lat, lim, x, blocks):
    r = oracle.Sdm(lib, f[1], f[3], f[4], depth, K, lat, lim)
    o = oracle.sdm(f[1], f[3], f[4], depth, K, lat, lim)
    pos = 0
    for b in blocks:
        blk = x[pos:pos + b]
        pos += b
        assert np.array_equal(r.process(blk), o.process(blk))
    assert np.array_equal(r.drain(4096), o.drain(4096))
    assert r.info() == o.info()


def test_sdm_restatement_equals_reference_random(ref, wide, oracle):
    t = _table(ref, oracle)
    rng = np.random.default_rng(2024)
    for trial in range(60):
        f = t[rng.integers(len(t))]
        K = int(rng.choice([1, 2, 3, 4, 8, 16, 31, 32]))
        depth = int(rng.choice([1, 2, 4, 8, 16, 31, 32, 33, 48, 64]))
        lat = int(rng.choice([1, 7, 16, 32, 33, 64, 128, 256]))
        lim = float(rng.choice([0.0, 0.0, 2.0, 10.0]))
        n = int(rng.integers(300, 5000))
        x = sdm_input(n, int(rng.integers(1 << 30)), amp=float(rng.choice([0.1, 0.4, 0.7])))
        blocks = []
        while sum(blocks) < n:
            blocks.append(int(rng.integers(1, 1500)))
        _cmp(oracle, wide if depth > 32 else ref, f, depth, K, lat, lim, x, blocks)


def test_sdm_long_latencies_equal_reference(ref, wide, oracle):
    """Traceback latencies above 256 up to SDM_TRELLIS_MAX_LAT = 2048
    (include/trellis.h:13, the plugin's range 16-2048, src/config.c:509-510)."""
    t = _table(ref, oracle)
    rng = np.random.default_rng(77)
    for lat, K, depth in [(257, 32, 64), (300, 2, 4), (777, 16, 32), (1024, 5, 48), (2048, 32, 32)]:
        f = t[rng.integers(len(t))]
        x = sdm_input(lat + 3000, int(rng.integers(1 << 30)), amp=0.5)
        blocks = [int(rng.integers(1, lat + 500)) for _ in range(8)]
        _cmp(oracle, wide if depth > 32 else ref, f, depth, K, lat, 0.0, x, blocks)


def test_sdm_k32_long_runs(ref, wide, oracle):
    """K = 32 over long inputs, where the act[32] store lands on path_hash[0]."""
    t = {(e[0], e[2]): e for e in _table(ref, oracle)}
    f = t[("clans-7", 5644800)]
    for depth, lat in [(8, 32), (16, 128), (32, 128), (64, 128)]:
        x = multitone(60000, depth + lat)
        _cmp(oracle, wide if depth > 32 else ref, f, depth, 32, lat, 0.0, x, [60000])


def test_widened_build_equals_narrow_at_depth_le_32(ref, wide, oracle):
    t = _table(ref, oracle)
    rng = np.random.default_rng(7)
    for _ in range(12):
        f = t[rng.integers(len(t))]
        depth = int(rng.choice([4, 16, 32]))
        x = sdm_input(6000, int(rng.integers(1 << 30)))
        a = oracle.Sdm(ref, f[1], f[3], f[4], depth, 32, 64).process(x)
        b = oracle.Sdm(wide, f[1], f[3], f[4], depth, 32, 64).process(x)
        assert np.array_equal(a, b)


def test_copy_seed_segment_equal_reference(ref, oracle):
    t = {(e[0], e[2]): e for e in _table(ref, oracle)}
    f = t[("clans-6", 5644800)]
    x = multitone(40000, 3)
    r0 = oracle.Sdm(ref, f[1], f[3], f[4], 32, 32, 128)
    o0 = oracle.sdm(f[1], f[3], f[4], 32, 32, 128)
    r0.process(x[:7000])
    o0.process(x[:7000])
    seed = r0.best_state()
    assert np.array_equal(seed, o0.best_state())
    for disc in (0, 100, 8192 - 128, 50000):
        r = oracle.Sdm(ref, f[1], f[3], f[4], 32, 32, 128)
        o = oracle.sdm(f[1], f[3], f[4], 32, 32, 128)
        r.copy_from(r0)
        o.copy_from(o0)
        r.seed(seed)
        o.seed(seed)
        assert np.array_equal(r.segment(x[7000:], disc), o.segment(x[7000:], disc))
        assert r.info() == o.info()


def test_estimator_equals_reference(ref, oracle):
    t = _table(ref, oracle)
    rng = np.random.default_rng(5)
    for _ in range(10):
        f = t[rng.integers(len(t))]
        x = multitone(20000, int(rng.integers(1000)))
        init = rng.standard_normal(f[1]) * 0.1
        for levels in (2, 16):
            for lim in (0.0, 1.5):
                a = oracle.estimate_state(f[1], f[3], f[4], init, x, lim, levels, lib=ref)
                b = oracle.estimate_state(f[1], f[3], f[4], init, x, lim, levels)
                assert np.array_equal(a, b)


def test_reference_init_limits_and_counts(ref, wide, oracle):
    """test/test_trellis.c:40-118: limits, +-1 output, count = N - lat, drain = lat."""
    t = _table(ref, oracle)
    f = t[0]
    for depth, K, lat in [(33, 16, 64), (8, 33, 64), (8, 16, 2049), (0, 16, 64)]:
        with pytest.raises(ValueError):
            oracle.Sdm(ref, f[1], f[3], f[4], depth, K, lat)
    o = oracle.sdm(f[1], f[3], f[4], 8, 16, 64)
    y = o.process(np.full(128, 0.5))
    assert len(y) == 64 and set(np.unique(y)) <= {-1.0, 1.0}
    o2 = oracle.sdm(f[1], f[3], f[4], 8, 16, 64)
    assert len(o2.process(np.zeros(64))) == 0
    assert len(o2.drain(256)) == 64


def test_packers_equal_reference(ref, oracle):
    rng = np.random.default_rng(11)
    L = ref.lib
    for n in (0, 7, 16, 33, 1000):
        for phase in (0, 1):
            bits = (rng.random(n) > 0.5).astype(np.uint8)
            fl = np.where(bits > 0, 1.0, -1.0).astype(np.float32)
            want = np.zeros(max(n // 16 * 3, 1), np.uint8)
            wph = L.ref_dop_pack_i24(fl.ctypes.data_as(oracle._fp), want.ctypes.data_as(oracle._u8p),
                                     n, phase)
            got, ph = oracle.dop_pack_bits(bits, phase)
            assert ph == wph
            assert np.array_equal(got, want[: n // 16 * 3])
            wb = np.zeros(max((n + 7) // 8, 1), np.uint8)
            L.ref_bits_pack(fl.ctypes.data_as(oracle._fp), wb.ctypes.data_as(oracle._u8p), n)
            assert np.array_equal(oracle.bits_pack(bits), wb[: (n + 7) // 8])


def test_dop_unpack_matches_reference(oracle):
    """The oracle's DoP unpack equals the reference's own dop_unpack, and the
    DoP float frames built from decisions unpack back to them."""
    ref = oracle.ref_lib()
    if ref is None:
        pytest.skip("reference sources absent")
    rng = np.random.default_rng(4)
    bits = (rng.random(16 * 5000) > 0.5).astype(np.uint8)
    for phase in (0, 1):
        pcm = oracle.dop_float_frames(bits, phase)
        mine = oracle.dop_unpack(pcm)
        theirs = oracle.dop_unpack(pcm, lib=ref)
        assert np.array_equal(mine, theirs)
        assert np.array_equal((mine > 0).astype(np.uint8), bits)


def test_samerate_boxcar_restatement(oracle):
    """Boxcar over +-1 decisions: an exact windowed count times 1/taps times
    the gain ramp, with the ring carried across blocks."""
    rng = np.random.default_rng(5)
    bits = np.where(rng.random(3000) > 0.5, 1.0, -1.0).astype(np.float32)
    taps = 64
    bc = oracle.Boxcar(taps)
    a = bc.process(bits[:1000], 0.0, 0.5)
    b = bc.process(bits[1000:], 0.5, 0.25)
    s = np.concatenate([np.zeros(taps - 1), bits.astype(np.float64)])
    win = np.array([s[i:i + taps].sum() for i in range(len(bits))])
    ga = 0.5 + 0.0 * np.arange(1000)
    gb = 0.5 + (0.25 - 0.5) / 1999 * np.arange(2000)
    np.testing.assert_allclose(a, win[:1000] / taps * ga, rtol=0, atol=1e-15)
    np.testing.assert_allclose(b, win[1000:] / taps * gb, rtol=0, atol=1e-15)


@pytest.mark.parametrize("name,rate,limit", [("clans-5", 2822400, 0.0), ("clans-7", 5644800, 0.0),
                                             ("clans-8", 11289600, 0.0), ("sdm-6", 5644800, 4.0)])
def test_precorr_matches_reference(oracle, name, rate, limit):
    """The PreCorr restatement (table training and decisions) equals the
    reference's src/precorr.c bit for bit, streamed."""
    if oracle.ref_lib() is None:
        pytest.skip("reference sources absent")
    from foo_dsd_trellis_gb300 import ntf
    f = ntf.get_filter(name, rate)
    mine = oracle.PreCorr(f.order, np.array(f.a), np.array(f.g), limit)
    ref = oracle.PreCorr(f.order, np.array(f.a), np.array(f.g), limit, ref=True)
    assert np.array_equal(mine.table().view(np.uint32), ref.table().view(np.uint32))
    x = 0.6 * multitone(30000, 3)
    for lo, hi in ((0, 7), (7, 20000), (20000, 30000)):
        assert np.array_equal(mine.process(x[lo:hi]), ref.process(x[lo:hi]))
