"""Failure paths of the device code, made to happen without a fault: the
kernels' bounded waits and walks are shortened (DSDGPU_OPT_FAILURE_TEST) so
that they run out, the call must return DSDGPU_ERR_DEVICE from the status
word, and the same context must then convert correctly again.  Nothing here
hangs or faults the GPU: every wait has an iteration or clock limit, and the
part queue's missing entry only delays the one warp that takes it by ~1 ms."""
import numpy as np
import pytest

from signals import multitone

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _ntf(name, rate):
    from foo_dsd_trellis_gb300 import ntf
    return ntf.get_filter(name, rate)


def test_part_queue_wait_gives_up_and_context_recovers():
    """A balanced launch whose part queue holds one entry that no part
    publishes: the warp that takes it gives up after the shortened wait, the
    call reports DSDGPU_ERR_DEVICE, and the next call on the same context
    equals the one-segment-per-warp launch."""
    from foo_dsd_trellis_gb300 import _lib
    from foo_dsd_trellis_gb300.das import DasChannels
    f = _ntf("clans-7", 6144000)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    pipes = 4 * sms
    S = (pipes + pipes // 20) // 2 + 1            # segments per channel, 2 channels
    seg = 20000
    x = np.stack([multitone(S * seg, 30) * 1.6, multitone(S * seg, 31) * 1.3])
    fir = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    d = DasChannels(f.order, f.a, f.g, 16, 32, 32, num_channels=2)
    _lib.check(d.h, d.L.dsdgpu_set_option(d.h, _lib.OPT_FAILURE_TEST, _lib.FAIL_PART_WAIT))
    with pytest.raises(_lib.DsdGpuError) as err:
        d.process_chunk(fir, nsegs=S, seed_mode=0)
    assert err.value.code == _lib.ERR_DEVICE
    assert d.last_sdm_kernel() == "sdm_parts_kernel<7>"
    _lib.check(d.h, d.L.dsdgpu_set_option(d.h, _lib.OPT_FAILURE_TEST, 0))
    d.L.dsdgpu_sdm_reset(d.h, -1)
    got, seams = d.process_chunk(fir, nsegs=S, seed_mode=0)
    d.close()
    plain = DasChannels(f.order, f.a, f.g, 16, 32, 32, num_channels=2)
    _lib.check(plain.h, plain.L.dsdgpu_set_option(plain.h, _lib.OPT_SDM_BALANCE, 0))
    want, wseams = plain.process_chunk(fir, nsegs=S, seed_mode=0)
    plain.close()
    assert list(seams) == list(wseams)
    assert torch.equal(got, want)


def test_chain_walk_bound_gives_up_and_context_recovers(oracle):
    """The serial selection's path-hash chain walk (src/trellis.c:668-700 in the
    reference's order) bounded to one hop: a trellis with many colliding
    paths in a bucket (K = 32, depth 64: 64 children over the 128 buckets of
    their low path bits, the recent decisions that survivors mostly share)
    reports DSDGPU_ERR_DEVICE; after the option is cleared and the contexts
    reset, the same input gives the oracle's bits."""
    from foo_dsd_trellis_gb300 import _lib
    from foo_dsd_trellis_gb300.sdm import TrellisSdm
    f = _ntf("clans-7", 6144000)
    K, depth, lat = 32, 64, 64
    x = np.stack([multitone(20000, 41) * 2.0, multitone(20000, 42) * 2.0])
    g = TrellisSdm(f.order, f.a, f.g, depth, K, lat, num_contexts=2)
    g.set_select(_lib.SELECT_EXACT)
    g.set_option(_lib.OPT_FAILURE_TEST, _lib.FAIL_CHAIN_WALK)
    with pytest.raises(_lib.DsdGpuError) as err:
        g.process_block(torch.from_numpy(x).cuda())
    assert err.value.code == _lib.ERR_DEVICE
    g.set_option(_lib.OPT_FAILURE_TEST, 0)
    _lib.check(g.h, g.L.dsdgpu_sdm_reset(g.h, -1))
    got = [t.cpu().numpy() for t in g.process_block(torch.from_numpy(x).cuda())]
    g.close()
    for c in range(2):
        ref = oracle.sdm(f.order, np.array(f.a), np.array(f.g), depth, K, lat)
        assert np.array_equal(got[c], oracle.sdm_bits(ref, x[c]))


def test_failure_test_option_rejects_unknown_bits():
    from foo_dsd_trellis_gb300 import _lib
    from foo_dsd_trellis_gb300.sdm import TrellisSdm
    f = _ntf("clans-6", 5644800)
    g = TrellisSdm(f.order, f.a, f.g, 8, 4, 16, num_contexts=1)
    assert g.L.dsdgpu_set_option(g.h, _lib.OPT_FAILURE_TEST, 4) == _lib.ERR_ARG
    g.close()
