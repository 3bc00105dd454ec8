"""The allocation-free SDM entry point (dsdgpu_sdm_process_noalloc), called
through the C ABI, against the regular entry point (dsdgpu_sdm_process on a
freshly set-up context).  It exists for callers that cannot allocate device
memory (a real-time audio callback, a fixed device-memory budget); its
scratch is a fixed device array shared by all calls, so two calls in a row
check that the second does not see the first one's leftovers.  Decisions are
bits, so the tolerance is exact equality, as in the other SDM tests.  This
file is collected last on purpose."""
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


def _noalloc(L, p, x):
    nch, n = x.shape
    out = torch.full((nch, n), 7, dtype=torch.uint8, device=x.device)
    oc = (C.c_size_t * nch)()
    torch.cuda.synchronize()
    rc = L.dsdgpu_sdm_process_noalloc(C.byref(p), nch, C.c_void_p(x.data_ptr()), n, n,
                                      C.c_void_p(out.data_ptr()), n, oc, None)
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


def test_noalloc_rejects_more_channels_than_its_scratch():
    from foo_dsd_trellis_gb300 import _lib, ntf
    L = _lib.load()
    f = ntf.get_filter("clans-5", ntf.DSD_RATE_64)
    p = _params(f, 16, 8, 32)
    x = torch.zeros((9, 100), dtype=torch.float64, device="cuda")
    out = torch.zeros((9, 100), dtype=torch.uint8, device="cuda")
    rc = L.dsdgpu_sdm_process_noalloc(C.byref(p), 9, C.c_void_p(x.data_ptr()), 100, 100,
                                      C.c_void_p(out.data_ptr()), 100, None, None)
    assert rc == _lib.ERR_TOO_LARGE
