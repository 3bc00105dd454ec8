"""GPU trellis SDM vs the oracle (bit-exact): the CUDA path is called through
the C ABI (libdsdgpu.so via foo_dsd_trellis_gb300.sdm) and compared decision
by decision with the CPU restatement of src/trellis.c."""
import zlib

import numpy as np
import pytest

from signals import multitone, sdm_input

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _ntf(name, rate):
    from foo_dsd_trellis_gb300 import ntf
    return ntf.get_filter(name, rate)


def _gpu_sdm(f, depth, K, lat, lim=0.0, nctx=1):
    from foo_dsd_trellis_gb300.sdm import TrellisSdm
    return TrellisSdm(f.order, f.a, f.g, depth, K, lat, lim, num_contexts=nctx)


def _ora(oracle, f, depth, K, lat, lim=0.0):
    return oracle.sdm(f.order, np.array(f.a), np.array(f.g), depth, K, lat, lim)


CASES = [
    # (ntf name, rate, depth, K, lat, limit)
    ("clans-5", 2822400, 32, 16, 32, 0.0),     # the plain DSD64 configuration
    ("clans-7", 6144000, 64, 32, 128, 0.0),    # the DSD128 DAS configuration
    ("clans-6", 5644800, 32, 32, 128, 0.0),
    ("clans-8", 11289600, 48, 16, 32, 0.0),
    ("sdm-6", 22579200, 16, 2, 32, 10.0),
    ("clans-4", 2822400, 8, 32, 64, 4.0),
    ("sdm-8", 5644800, 4, 8, 16, 0.0),
    ("clans-6", 2822400, 1, 3, 7, 0.0),
    ("sdm-5", 11289600, 33, 31, 100, 2.0),
    ("clans-6", 2822400, 32, 1, 256, 0.0),
]


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-d{c[2]}-K{c[3]}-lat{c[4]}" for c in CASES])
def test_process_block_bit_exact(oracle, case):
    name, rate, depth, K, lat, lim = case
    f = _ntf(name, rate)
    n = 20000
    x = sdm_input(n, seed=zlib.crc32(repr(case).encode()) & 0xffff, amp=0.45)
    ref = _ora(oracle, f, depth, K, lat, lim)
    want = oracle.sdm_bits(ref, x)
    g = _gpu_sdm(f, depth, K, lat, lim)
    got = g.process_block(torch.from_numpy(x).cuda())[0].cpu().numpy()
    assert len(got) == len(want) == n - lat
    bad = np.nonzero(got != want)[0]
    assert bad.size == 0, f"first mismatch at {bad[:5]} of {len(want)}"
    q = g.query(0)
    info = ref.info()
    assert q["num_cands"] == info["num_cands"]
    assert q["total_children"] == info["total_children"]
    assert q["next_filter_drops"] == info["next_filter_drops"]
    assert q["conv_fail"] == info["conv_fail"]
    np.testing.assert_array_equal(q["best_state"], ref.best_state())


def test_streaming_blocks_and_drain(oracle):
    f = _ntf("clans-7", 6144000)
    x = multitone(30000, seed=5)
    ref = _ora(oracle, f, 64, 32, 128)
    g = _gpu_sdm(f, 64, 32, 128)
    rng = np.random.default_rng(3)
    pos = 0
    while pos < len(x):
        b = int(rng.integers(1, 5000))
        blk = x[pos:pos + b]
        pos += b
        want = oracle.sdm_bits(ref, blk)
        got = g.process_block(torch.from_numpy(blk).cuda())[0].cpu().numpy()
        np.testing.assert_array_equal(got, want)
    want = (ref.drain(500) > 0).astype(np.uint8)
    got = g.drain(500)[0].cpu().numpy()
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("K,depth,lat,lim", [(32, 64, 257, 0.0), (32, 32, 2048, 0.0),
                                             (16, 48, 1000, 2.0), (2, 4, 512, 0.0),
                                             (5, 16, 300, 0.0)])
def test_long_latency_streaming_and_drain(oracle, K, depth, lat, lim):
    """Latencies above 256 (up to the reference's 2048) take the wide-ring
    kernel: ragged streamed blocks over two channels, then drain."""
    f = _ntf("clans-7", 5644800)
    nch = 2
    xs = [sdm_input(lat + 9000, seed=lat + c, amp=0.5) for c in range(nch)]
    refs = [_ora(oracle, f, depth, K, lat, lim) for _ in range(nch)]
    g = _gpu_sdm(f, depth, K, lat, lim, nctx=nch)
    rng = np.random.default_rng(lat)
    pos = 0
    n = len(xs[0])
    while pos < n:
        b = min(int(rng.integers(1, 2 * lat)), n - pos)
        blk = np.stack([x[pos:pos + b] for x in xs])
        pos += b
        got = g.process_block(torch.from_numpy(blk).cuda())
        for c in range(nch):
            np.testing.assert_array_equal(got[c].cpu().numpy(), oracle.sdm_bits(refs[c], blk[c]))
    got = g.drain(lat + 10, 0, nch)
    for c in range(nch):
        want = (refs[c].drain(lat + 10) > 0).astype(np.uint8)
        assert len(want) == lat
        np.testing.assert_array_equal(got[c].cpu().numpy(), want)
    q = g.query(1)
    np.testing.assert_array_equal(q["best_state"], refs[1].best_state())


def test_short_block_then_drain(oracle):
    """Fewer samples than the latency, then drain (test/test_trellis.c:122-140)."""
    f = _ntf("clans-5", 2822400)
    ref = _ora(oracle, f, 8, 16, 64)
    g = _gpu_sdm(f, 8, 16, 64)
    x = np.zeros(40)
    assert len(oracle.sdm_bits(ref, x)) == 0
    assert g.process_block(torch.from_numpy(x).cuda())[0].numel() == 0
    want = (ref.drain(256) > 0).astype(np.uint8)
    got = g.drain(256)[0].cpu().numpy()
    assert len(want) == 40
    np.testing.assert_array_equal(got, want)


def test_multichannel_and_host_form(oracle):
    f = _ntf("clans-6", 5644800)
    xs = np.stack([sdm_input(8000, seed=s) for s in (1, 2, 3)])
    g = _gpu_sdm(f, 32, 32, 128, nctx=3)
    got = g.process_block_host(xs)
    for c in range(3):
        ref = _ora(oracle, f, 32, 32, 128)
        want = ref.process(xs[c])
        np.testing.assert_array_equal(got[c], want)


def test_segments_copy_seed_discard(oracle):
    """DAS-style segments: copy a warmed context, seed the candidates with a
    state, run with warm-up discard (src/engine.c:915-938)."""
    f = _ntf("clans-7", 6144000)
    K, depth, lat = 32, 64, 128
    x = multitone(60000, seed=11)
    base = _ora(oracle, f, depth, K, lat)
    oracle.sdm_bits(base, x[:5000])
    g = _gpu_sdm(f, depth, K, lat, nctx=5)
    g.process_block(torch.from_numpy(x[:5000]).cuda(), first=0)
    g.copy_state(4, 0)          # snapshot: segments must not read a context that runs
    seed = np.array(base.best_state())
    from foo_dsd_trellis_gb300.sdm import SegmentSpec
    specs, wants = [], []
    for i, (a, b, disc, sd) in enumerate([(5000, 20000, 0, False), (15000, 32000, 3000, True),
                                          (28000, 45000, 8192 - lat, True),
                                          (40000, 60000, 100000, False)]):
        ctxo = oracle.sdm(f.order, np.array(f.a), np.array(f.g), depth, K, lat)
        ctxo.copy_from(base)
        if sd:
            ctxo.seed(seed)
        wants.append(oracle.segment_bits(ctxo, x[a:b], disc))
        specs.append(SegmentSpec(torch.from_numpy(x[a:b].copy()).cuda(), channel=i,
                                 discard=disc, seed_from=4,
                                 seed_state=torch.from_numpy(seed).cuda() if sd else None))
    # channel 0 is also a target: copy_state of 4 onto 0 is the seeding source
    outs = g.segments(specs)
    for got, want in zip(outs, wants):
        np.testing.assert_array_equal(got.cpu().numpy(), want)


VERIFY_CASES = CASES + [
    ("clans-7", 6144000, 64, 32, 128, 0.0),
    ("clans-7", 6144000, 32, 32, 64, 0.0),
    ("clans-6", 5644800, 16, 32, 32, 0.0),
    ("sdm-7", 5644800, 8, 32, 128, 3.0),
]


@pytest.mark.parametrize("case", VERIFY_CASES,
                         ids=[f"v-{c[0]}-d{c[2]}-K{c[3]}-lat{c[4]}-{i}" for i, c in enumerate(VERIFY_CASES)])
def test_fast_selection_verified_against_serial(oracle, case):
    """Verify mode runs the serial (reference-order) selection every sample
    and checks the parallel one against it: any disagreement in survivors,
    order, costs, hashed set or stored chain links fails the call."""
    from foo_dsd_trellis_gb300 import _lib
    name, rate, depth, K, lat, lim = case
    f = _ntf(name, rate)
    x = multitone(40000, seed=zlib.crc32(repr(case).encode()) & 0xffff) * 1.5
    g = _gpu_sdm(f, depth, K, lat, lim, nctx=2)
    g.set_select(_lib.SELECT_VERIFY)
    got = g.process_block(torch.from_numpy(x).cuda())[0].cpu().numpy()
    want = oracle.sdm_bits(_ora(oracle, f, depth, K, lat, lim), x)
    assert np.array_equal(got, want)
    # seeded segments start with equal costs everywhere (ties)
    from foo_dsd_trellis_gb300.sdm import SegmentSpec
    seed = torch.from_numpy(np.array(g.query(0)["best_state"])).cuda()
    g.segments([SegmentSpec(torch.from_numpy(x[:20000].copy()).cuda(), channel=1, discard=300,
                            seed_from=0, seed_state=seed)])


def test_exact_and_fast_modes_agree(oracle):
    from foo_dsd_trellis_gb300 import _lib
    f = _ntf("clans-7", 6144000)
    x = multitone(30000, seed=77)
    outs = []
    for mode in (_lib.SELECT_FAST, _lib.SELECT_EXACT):
        g = _gpu_sdm(f, 64, 32, 128)
        g.set_select(mode)
        outs.append(g.process_block(torch.from_numpy(x).cuda())[0].cpu().numpy())
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("K,depth,lat,lim", [(2, 4, 128, 0.0), (1, 8, 32, 0.0), (2, 2, 200, 3.0),
                                             (4, 8, 32, 0.0), (3, 6, 64, 2.0), (4, 3, 100, 0.0)])
def test_small_k_streaming_channels_and_drain(oracle, K, depth, lat, lim):
    """Small trellises (K <= 4, including the reference's default K = 4,
    depth 8, lat 32) take the lane-split kernel: streamed blocks over several
    channels, short path masks (dedup on most samples), the limiter and the
    drain, against the oracle."""
    f = _ntf("clans-6", 5644800)
    nch = 5
    x = np.stack([multitone(12000, seed=40 + c) * (0.6 + 0.1 * c) for c in range(nch)])
    refs = [_ora(oracle, f, depth, K, lat, lim) for _ in range(nch)]
    g = _gpu_sdm(f, depth, K, lat, lim, nctx=nch)
    for lo, hi in ((0, 1), (1, 77), (77, 5000), (5000, 12000)):
        got = g.process_block(torch.from_numpy(np.ascontiguousarray(x[:, lo:hi])).cuda())
        for c in range(nch):
            np.testing.assert_array_equal(got[c].cpu().numpy(), oracle.sdm_bits(refs[c], x[c, lo:hi]))
    tail = g.drain(lat + 10, 0, nch)
    for c in range(nch):
        np.testing.assert_array_equal(tail[c].cpu().numpy(), (refs[c].drain(lat + 10) > 0).astype(np.uint8))
        q, info = g.query(c), refs[c].info()
        assert (q["num_cands"], q["total_children"], q["next_filter_drops"], q["conv_fail"]) == \
            (info["num_cands"], info["total_children"], info["next_filter_drops"], info["conv_fail"])
        np.testing.assert_array_equal(q["best_state"], refs[c].best_state())


@pytest.mark.parametrize("K,depth", [(2, 4), (4, 8), (1, 6)])
def test_kernels_share_the_context_format(oracle, K, depth):
    """One context carried through every SDM kernel in turn: the per-thread
    kernel (more jobs than the split kernel's cap), the lane-split kernel (few
    jobs), the warp kernel at 2 and 32 lanes (DSDGPU_OPT_SDM_LANES), then the
    split kernel again, each call continuing the previous one's state."""
    from foo_dsd_trellis_gb300 import _lib
    f = _ntf("clans-6", 5644800)
    many = 2600          # above the split kernel's 2 x 2 x 4 x 152 jobs (K <= 2)
    g = _gpu_sdm(f, depth, K, 32, 0.0, nctx=many)
    refs = [_ora(oracle, f, depth, K, 32) for _ in range(2)]
    x = np.stack([multitone(15000, seed=90 + c) * 0.7 for c in range(2)])
    pos = 0
    for stage, ln in (("all", 3000), ("split", 2500), ("lanes2", 3100), ("lanes32", 2900),
                      ("split", 3500)):
        blk = x[:, pos:pos + ln]
        pos += ln
        if stage == "all":
            if K > 2:
                continue
            xa = np.zeros((many, ln))
            xa[:2] = blk
            got = g.process_block(torch.from_numpy(xa).cuda())[:2]
        else:
            g.set_option(_lib.OPT_SDM_LANES, {"split": 0, "lanes2": 2, "lanes32": 32}[stage])
            got = g.process_block(torch.from_numpy(np.ascontiguousarray(blk)).cuda())
        for c in range(2):
            np.testing.assert_array_equal(got[c].cpu().numpy(), oracle.sdm_bits(refs[c], blk[c]),
                                          err_msg=stage)
    g.set_option(_lib.OPT_SDM_LANES, 0)
    got = g.drain(64, 0, 2)
    for c in range(2):
        np.testing.assert_array_equal(got[c].cpu().numpy(), (refs[c].drain(64) > 0).astype(np.uint8))


def test_small_k_many_jobs_take_the_per_thread_kernel(oracle):
    """More K <= 2 jobs than the lane-split kernel keeps resident (2,600
    channels of one launch) run one job per thread; every channel equals the
    oracle."""
    f = _ntf("clans-6", 5644800)
    nch, n = 2600, 300
    rng = np.random.default_rng(77)
    x = (rng.standard_normal((nch, n)) * 0.25).astype(np.float64)
    g = _gpu_sdm(f, 4, 2, 16, 0.0, nctx=nch)
    got = g.process_block(torch.from_numpy(x).cuda())
    for c in range(0, nch, 97):
        ref = _ora(oracle, f, 4, 2, 16)
        np.testing.assert_array_equal(got[c].cpu().numpy(), oracle.sdm_bits(ref, x[c]))


@pytest.mark.parametrize("order", [2, 3, 9, 10])
@pytest.mark.parametrize("K", [2, 8])
def test_orders_outside_the_table(oracle, order, K):
    """Orders 2, 3, 9 and 10 (accepted by the ABI, absent from the NTF table;
    a real NTF truncated or zero-padded), through the small-trellis and warp
    kernels."""
    src = _ntf("clans-4", 2822400) if order <= 4 else _ntf("clans-8", 11289600)
    a, g = np.zeros(order), np.zeros(order)
    m = min(order, src.order)
    a[:m], g[:m] = np.array(src.a[:m]), np.array(src.g[:m])

    class F:
        pass
    f = F()
    f.order, f.a, f.g = order, list(a), list(g)
    x = sdm_input(6000, seed=order * 10 + K, amp=0.3)
    ref = oracle.sdm(order, a, g, 16, K, 24, 0.0)
    want = oracle.sdm_bits(ref, x)
    gpu = _gpu_sdm(f, 16, K, 24)
    got = gpu.process_block(torch.from_numpy(x).cuda())[0].cpu().numpy()
    np.testing.assert_array_equal(got, want)


def test_estimate_state_batch(oracle):
    """dsdgpu_sdm_estimate_state (sdm_estimate_state_multibit, src/trellis.c:1125-1187)
    over many inputs in one launch equals the oracle (pinned to the reference's
    compiled estimator), for orders 2..10, 2/3/16/97/2000 levels (the quantiser
    index from reciprocal products, its table, and the exact divisions), the limiter and
    counts 0, 1 and 20,000."""
    import ctypes as C
    from foo_dsd_trellis_gb300 import _lib, ntf
    from signals import multitone
    L = _lib.load()
    h = C.c_void_p()
    assert L.dsdgpu_create(0, C.byref(h)) == 0
    rng = np.random.default_rng(11)
    names = ["clans-4", "clans-5", "clans-6", "clans-7", "clans-8", "sdm-5", "sdm-8"]
    for levels in (2, 3, 16, 97, 2000):
        for lim in (0.0, 1.5):
            for name in names:
                f = ntf.get_filter(name, 5644800)
                p = _lib.SdmParams()
                p.order = f.order
                for i in range(f.order):
                    p.a[i], p.g[i] = f.a[i], f.g[i]
                p.state_limit = lim
                counts = [0, 1, 20000, 777]
                xs = [multitone(max(n, 1), int(rng.integers(1000))) * 0.5 for n in counts]
                d_x = [torch.from_numpy(x).cuda() for x in xs]
                items = (_lib.EstimateItem * len(counts))()
                inits = []
                for j, n in enumerate(counts):
                    items[j].d_in = d_x[j].data_ptr()
                    items[j].count = n
                    init = rng.standard_normal(f.order) * 0.1
                    inits.append(init)
                    for k in range(f.order):
                        items[j].init_state[k] = init[k]
                _lib.check(h, L.dsdgpu_sdm_estimate_state(h, C.byref(p), levels, items, len(counts)))
                for j, n in enumerate(counts):
                    want = oracle.estimate_state(f.order, np.array(f.a), np.array(f.g), inits[j],
                                                 xs[j][:n], lim, levels)
                    got = np.array(items[j].out_state[: f.order])
                    assert np.array_equal(got, want), (name, levels, lim, n)
    p = _lib.SdmParams()
    p.order = 1
    assert L.dsdgpu_sdm_estimate_state(h, C.byref(p), 16, None, 0) == _lib.ERR_ARG
    p.order = 7
    assert L.dsdgpu_sdm_estimate_state(h, C.byref(p), 1, None, 0) == _lib.ERR_ARG
    L.dsdgpu_destroy(h)


def test_estimate_state_level_boundaries(oracle):
    """The estimator's quantiser at its level boundaries: from a zero state
    the first output is v = x + a0 * x, so first inputs placed on, and one or
    a few ulps and 1e-12 .. 1e-9 either side of, every boundary
    (v / a0 + 1) / step + 0.5 = k (and x = 0, where u = 7.5 exactly at 16
    levels) reach the samples the warp form hands to the reference's
    divisions; the next 40 inputs continue from the state they leave.  Equal
    to the oracle for 3, 16 and 32 levels, with and without the limiter."""
    import ctypes as C
    from foo_dsd_trellis_gb300 import _lib, ntf
    L = _lib.load()
    h = C.c_void_p()
    assert L.dsdgpu_create(0, C.byref(h)) == 0
    f = ntf.get_filter("clans-7", 5644800)
    a0 = float(f.a[0])
    rng = np.random.default_rng(5)
    for levels in (3, 16, 32):
        step = 2.0 / (levels - 1)
        firsts = [0.0]
        for k in range(levels + 1):
            yi = (k - 0.5) * step - 1.0
            x0 = yi * a0 / (1.0 + a0)
            firsts.append(x0)
            for d in (1, 2, 4):
                firsts.append(float(np.nextafter(x0, np.inf) if d == 1 else x0 + d * np.spacing(x0)))
                firsts.append(float(np.nextafter(x0, -np.inf) if d == 1 else x0 - d * np.spacing(x0)))
            for rel in (1e-12, 3e-10, 1e-9, 2e-9):
                firsts.extend([x0 * (1 + rel) + rel, x0 * (1 - rel) - rel])
        for lim in (0.0, 1.5):
            p = _lib.SdmParams()
            p.order = f.order
            for i in range(f.order):
                p.a[i], p.g[i] = f.a[i], f.g[i]
            p.state_limit = lim
            xs = [np.concatenate([[x0], 0.3 * rng.standard_normal(40)]) for x0 in firsts
                  for _ in range(2)]
            d_x = [torch.from_numpy(x).cuda() for x in xs]
            items = (_lib.EstimateItem * len(xs))()
            for j, x in enumerate(xs):
                items[j].d_in = d_x[j].data_ptr()
                items[j].count = len(x) if j % 2 else 1
            _lib.check(h, L.dsdgpu_sdm_estimate_state(h, C.byref(p), levels, items, len(xs)))
            for j, x in enumerate(xs):
                n = items[j].count
                want = oracle.estimate_state(f.order, np.array(f.a), np.array(f.g),
                                             np.zeros(f.order), x[:n], lim, levels)
                got = np.array(items[j].out_state[: f.order])
                assert np.array_equal(got, want), (levels, lim, j, x[0])
    L.dsdgpu_destroy(h)


def test_state_distance(oracle):
    """dsdgpu_sdm_state_distance (src/trellis.c:1094-1109) of two contexts run on
    different inputs equals the sum of squared differences of the oracle's best
    states, added in order."""
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.sdm import TrellisSdm
    from foo_dsd_trellis_gb300 import _lib
    import ctypes as C
    from signals import multitone
    f = ntf.get_filter("clans-7", 5644800)
    sdm = TrellisSdm(f.order, f.a, f.g, 16, 8, 32, 0.0, num_contexts=2)
    xs = [multitone(5000, 3 + c) * 0.6 for c in range(2)]
    refs = [oracle.sdm(f.order, np.array(f.a), np.array(f.g), 16, 8, 32) for _ in range(2)]
    sdm.process_block(torch.from_numpy(np.stack(xs)).cuda())
    for c in range(2):
        oracle.sdm_bits(refs[c], xs[c])
    d = C.c_double()
    _lib.check(sdm.h, sdm.L.dsdgpu_sdm_state_distance(sdm.h, 0, 1, C.byref(d)))
    sa, sb = refs[0].best_state(), refs[1].best_state()
    want = 0.0
    for i in range(f.order):
        t = sa[i] - sb[i]
        want += t * t
    assert d.value == want
    _lib.check(sdm.h, sdm.L.dsdgpu_sdm_state_distance(sdm.h, 1, 1, C.byref(d)))
    assert d.value == 0.0
    assert sdm.L.dsdgpu_sdm_state_distance(sdm.h, 0, 2, C.byref(d)) == _lib.ERR_ARG
    sdm.close()
