"""The allocation-free SDM entry point (dsdgpu_sdm_process_noalloc), called
through the C ABI.  It exists for callers that cannot allocate device memory:
a player's real-time audio callback, where an allocation can block on driver
locks and cause a dropout, and hosts with a fixed device-memory budget.  Its
scratch is a fixed device array shared by all calls, so every case runs two
calls in a row and checks that the second does not see the first one's
leftovers.  Decisions are bits, so the tolerance is exact equality, as in the
other SDM tests.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from signals import multitone, sdm_input

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _params(f, depth, K, lat):
    from foo_dsd_trellis_gb300 import _lib
    p = _lib.SdmParams()
    p.order = f.order
    for i in range(f.order):
        p.a[i] = f.a[i]
        p.g[i] = f.g[i]
    p.depth, p.cands, p.lat, p.state_limit = depth, K, lat, 0.0
    return p


def _noalloc(L, p, x, keep_state=0):
    nch, n = x.shape
    out = torch.full((nch, n), 7, dtype=torch.uint8, device=x.device)
    oc = (C.c_size_t * nch)()
    torch.cuda.synchronize()
    rc = L.dsdgpu_sdm_process_noalloc(C.byref(p), nch, keep_state, C.c_void_p(x.data_ptr()), n,
                                      n, C.c_void_p(out.data_ptr()), n, oc, None)
    assert rc == 0, rc
    return [out[c, : oc[c]].cpu().numpy() for c in range(nch)]


def _regular(f, depth, K, lat, x):
    from foo_dsd_trellis_gb300.sdm import TrellisSdm
    g = TrellisSdm(f.order, f.a, f.g, depth, K, lat, num_contexts=x.shape[0])
    got = [t.cpu().numpy() for t in g.process_block(x)]
    g.close()
    return got


def test_noalloc_matches_regular_entry_point_twice():
    from foo_dsd_trellis_gb300 import _lib, ntf
    L = _lib.load()
    f = ntf.get_filter("clans-7", ntf.DSD48_RATE_128)
    depth, K, lat = 64, 32, 128
    p = _params(f, depth, K, lat)
    first = torch.from_numpy(np.stack([sdm_input(12000, s) for s in (31, 32, 33)])).cuda()
    second = torch.from_numpy(np.stack([multitone(9000, s) for s in (41, 42)])).cuda()
    for x in (first, second):
        got = _noalloc(L, p, x)
        want = _regular(f, depth, K, lat, x)
        assert len(got) == len(want)
        for g, w in zip(got, want):
            assert len(g) == len(w) == x.shape[1] - lat
            assert np.array_equal(g, w)


@pytest.mark.parametrize("K,depth,lat", [(2, 4, 32), (4, 8, 64), (32, 64, 128), (8, 16, 512)],
                         ids=["K2", "K4", "K32", "K8_lat512"])
def test_noalloc_matches_oracle_streamed(oracle, K, depth, lat):
    """A fresh call and a continuing call (keep_state) equal the oracle's
    sdm_process_block over the two blocks in turn; then a fresh call again
    restarts the stream.  K <= 4 reaches the small-trellis kernels, lat 512 the
    wide-ring kernel."""
    from foo_dsd_trellis_gb300 import _lib, ntf
    L = _lib.load()
    f = ntf.get_filter("clans-6", 5644800)
    p = _params(f, depth, K, lat)
    x = np.stack([sdm_input(7000, s) for s in (51, 52)])
    blocks = [x[:, :3000], x[:, 3000:]]
    refs = [oracle.sdm(f.order, np.array(f.a), np.array(f.g), depth, K, lat) for _ in range(2)]
    for i, b in enumerate(blocks):
        got = _noalloc(L, p, torch.from_numpy(np.ascontiguousarray(b)).cuda(), keep_state=i)
        for c in range(2):
            want = oracle.sdm_bits(refs[c], b[c])
            assert len(got[c]) == len(want) == b.shape[1] - (lat if i == 0 else 0)
            assert np.array_equal(got[c], want)
    again = _noalloc(L, p, torch.from_numpy(np.ascontiguousarray(blocks[1])).cuda())
    fresh = oracle.sdm(f.order, np.array(f.a), np.array(f.g), depth, K, lat)
    assert np.array_equal(again[0], oracle.sdm_bits(fresh, blocks[1][0]))


def test_noalloc_allocates_nothing_after_warmup():
    """After one warm-up call (which may load the kernels), further calls,
    fresh or continuing, leave the device's free memory unchanged."""
    from foo_dsd_trellis_gb300 import _lib, ntf
    L = _lib.load()
    f = ntf.get_filter("clans-7", ntf.DSD48_RATE_128)
    p = _params(f, 64, 32, 128)
    x = torch.from_numpy(np.stack([sdm_input(6000, s) for s in (61, 62)])).cuda()
    out = torch.zeros((2, 6000), dtype=torch.uint8, device="cuda")
    oc = (C.c_size_t * 2)()
    args = (C.c_void_p(x.data_ptr()), 6000, 6000, C.c_void_p(out.data_ptr()), 6000, oc, None)
    assert L.dsdgpu_sdm_process_noalloc(C.byref(p), 2, 0, *args) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for keep in (1, 0, 1):
        assert L.dsdgpu_sdm_process_noalloc(C.byref(p), 2, keep, *args) == 0
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_bad_calls():
    """More channels than its scratch holds, overlapping rows, a continuing
    call whose parameters differ from the previous call's, a bad flag."""
    from foo_dsd_trellis_gb300 import _lib, ntf
    L = _lib.load()
    f = ntf.get_filter("clans-5", ntf.DSD_RATE_64)
    p = _params(f, 16, 8, 32)
    x = torch.zeros((9, 100), dtype=torch.float64, device="cuda")
    out = torch.zeros((9, 100), dtype=torch.uint8, device="cuda")
    xp, op = C.c_void_p(x.data_ptr()), C.c_void_p(out.data_ptr())
    assert L.dsdgpu_sdm_process_noalloc(C.byref(p), 9, 0, xp, 100, 100, op, 100, None,
                                        None) == _lib.ERR_TOO_LARGE
    assert L.dsdgpu_sdm_process_noalloc(C.byref(p), 2, 0, xp, 50, 100, op, 100, None,
                                        None) == _lib.ERR_ARG
    assert L.dsdgpu_sdm_process_noalloc(C.byref(p), 2, 0, xp, 100, 100, op, 10, None,
                                        None) == _lib.ERR_ARG
    assert L.dsdgpu_sdm_process_noalloc(C.byref(p), 2, 2, xp, 100, 100, op, 100, None,
                                        None) == _lib.ERR_ARG
    assert L.dsdgpu_sdm_process_noalloc(C.byref(p), 2, 0, xp, 100, 100, op, 100, None,
                                        None) == 0
    q = _params(f, 16, 4, 32)
    assert L.dsdgpu_sdm_process_noalloc(C.byref(q), 2, 1, xp, 100, 100, op, 100, None,
                                        None) == _lib.ERR_STATE
    assert L.dsdgpu_sdm_process_noalloc(C.byref(p), 3, 1, xp, 100, 100, op, 100, None,
                                        None) == _lib.ERR_STATE
    p.lat = 4096
    assert L.dsdgpu_sdm_process_noalloc(C.byref(p), 2, 0, xp, 100, 100, op, 100, None,
                                        None) == _lib.ERR_ARG
