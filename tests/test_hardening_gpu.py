"""Edge cases of the reference's engine hardening tests
(test/test_hardening.c:280-475, 548-562) on this path, through the C ABI:
zero-length calls, one-sample blocks, drain on a fresh or reset context,
many small blocks in a row (1,280 inputs at lat 64 give 1,216 decisions),
reset, and closing twice.  Decisions are compared with the oracle's trellis
(pinned to src/trellis.c) bit for bit."""
import ctypes as C

import numpy as np
import pytest

from signals import multitone, sdm_input

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

DSD64 = 2822400


def _f():
    from foo_dsd_trellis_gb300 import ntf
    return ntf.get_filter("clans-5", DSD64)


def _pair(oracle, depth=16, K=8, lat=64, nctx=1):
    from foo_dsd_trellis_gb300.sdm import TrellisSdm
    f = _f()
    g = TrellisSdm(f.order, f.a, f.g, depth, K, lat, num_contexts=nctx)
    refs = [oracle.sdm(f.order, np.array(f.a), np.array(f.g), depth, K, lat) for _ in range(nctx)]
    return g, refs


def test_zero_length_block_changes_nothing(oracle):
    """test_zero_length_block: an empty block returns no decisions, raises no
    error and leaves the stream where it was."""
    g, (ref,) = _pair(oracle)
    x = sdm_input(3000, 7, amp=0.5)
    empty = torch.zeros((1, 0), dtype=torch.float64, device="cuda")
    assert g.process_block(empty)[0].numel() == 0
    a = g.process_block(torch.from_numpy(x[:1000]).cuda())[0].cpu().numpy()
    assert g.process_block(empty)[0].numel() == 0
    b = g.process_block(torch.from_numpy(x[1000:]).cuda())[0].cpu().numpy()
    want = oracle.sdm_bits(ref, x)
    assert np.array_equal(np.concatenate([a, b]), want)
    g.close()


def test_empty_das_chunk_then_a_chunk(oracle):
    """An empty DAS chunk leaves the persistent contexts alone: the next chunk
    equals the oracle's DAS of that chunk on fresh contexts."""
    from foo_dsd_trellis_gb300.das import DasChannels
    f = _f()
    x = np.stack([multitone(60000, 31) * 1.5, multitone(60000, 32)])
    want, ws, _ = oracle.das_run(f.order, np.array(f.a), np.array(f.g), 16, 8, 32, 0.0, x,
                                 seg_len=8192, seed_mode=0)
    d = DasChannels(f.order, f.a, f.g, 16, 8, 32, num_channels=2)
    bits, _ = d.process_chunk(torch.zeros((2, 0), dtype=torch.float64, device="cuda"),
                              seg_len=8192)
    assert bits.shape[-1] == 0
    got, seams = d.process_chunk(torch.from_numpy(x).cuda(), seg_len=8192, seed_mode=0)
    assert list(seams) == list(ws)
    assert np.array_equal(got.cpu().numpy(), want)
    d.close()


def test_zero_length_fir_pack_das_pipeline():
    """Zero frames through the FIR chain, the packers, DAS and the whole path:
    no output, no error, and null buffers accepted for an empty call."""
    from foo_dsd_trellis_gb300 import _lib
    from foo_dsd_trellis_gb300.das import DasChannels
    from foo_dsd_trellis_gb300.fir import FirChain
    from foo_dsd_trellis_gb300.pack import Packer
    from foo_dsd_trellis_gb300.pipeline import Encoder
    fc = FirChain(44100, DSD64, num_channels=2)
    y = fc.process(torch.zeros((2, 0), dtype=torch.float32, device="cuda"))
    assert y.shape[-1] == 0
    fc.close()
    pk = Packer()
    frames, ph = pk.dop(torch.zeros((2, 0), dtype=torch.uint8, device="cuda"), phase=1)
    assert frames.shape[0] == 0 and ph == 1
    assert pk.native(torch.zeros((2, 0), dtype=torch.uint8, device="cuda")).shape[1] == 0
    pk.close()
    f = _f()
    d = DasChannels(f.order, f.a, f.g, 16, 8, 32, num_channels=2)
    bits, seams = d.process_chunk(torch.zeros((2, 0), dtype=torch.float64, device="cuda"),
                                  seg_len=8192)
    assert bits.shape[-1] == 0
    d.close()
    enc = Encoder(44100, DSD64, 2, f, 16, 8, 32, seg_len=8192)
    out = torch.zeros(64, dtype=torch.uint8, device="cuda")
    _, nbytes = enc.process(torch.zeros((2, 0), dtype=torch.float32, device="cuda"), out)
    assert nbytes == 0
    # the raw ABI with null buffers and a zero count, device and host forms
    ns, nb = C.c_size_t(7), C.c_size_t(7)
    assert enc.L.dsdgpu_pipeline_process(enc.h, None, 0, 0, 1.0, 1.0, None, 0, C.byref(ns),
                                         C.byref(nb)) == _lib.OK
    assert ns.value == 0 and nb.value == 0
    ns, nb = C.c_size_t(7), C.c_size_t(7)
    assert enc.L.dsdgpu_pipeline_process_host(enc.h, None, 0, 1.0, 1.0, None, 0, C.byref(ns),
                                              C.byref(nb)) == _lib.OK
    assert ns.value == 0 and nb.value == 0
    enc.close()


def test_single_sample_blocks(oracle):
    """test_single_sample_sdm, extended: one input per call for lat + 200
    samples; the first lat calls give nothing, then one decision each."""
    g, (ref,) = _pair(oracle, lat=32)
    x = sdm_input(232, 9, amp=0.5)
    got = []
    for i in range(len(x)):
        o = g.process_block(torch.from_numpy(x[i:i + 1]).cuda())[0].cpu().numpy()
        assert len(o) == (0 if i < 32 else 1)
        got.append(o)
    assert np.array_equal(np.concatenate(got), oracle.sdm_bits(ref, x))
    g.close()


def test_drain_without_processing(oracle):
    """test_drain_without_processing: a fresh context has nothing pending."""
    g, (ref,) = _pair(oracle)
    assert g.drain(128)[0].numel() == 0
    assert len(ref.drain(128)) == 0
    g.close()


def test_drain_after_reset(oracle):
    """test_drain_after_reset: 256 inputs, reset, drain: nothing comes out.
    The drain still steps the trellis over lat zero inputs and marks the
    context as draining (sdm_drain, src/trellis.c:1042-1062), so the next
    block equals the oracle's after the same calls, not a fresh context's."""
    g, (ref,) = _pair(oracle)
    x = 0.3 * np.sin(2 * np.pi * 1000.0 * np.arange(256) / DSD64)
    g.process_block(torch.from_numpy(x).cuda())
    oracle.sdm_bits(ref, x)
    g.reset()
    ref.reset()
    assert g.drain(128)[0].numel() == 0
    assert len(ref.drain(128)) == 0
    y = multitone(2000, 4)
    got = g.process_block(torch.from_numpy(y).cuda())[0].cpu().numpy()
    assert np.array_equal(got, oracle.sdm_bits(ref, y))
    g.close()


def test_reset_equals_fresh(oracle):
    """test_reset_then_different_signal: after a reset the context runs a new
    signal exactly as a fresh one does."""
    g, (ref,) = _pair(oracle)
    x = sdm_input(3000, 17, amp=0.5)
    g.process_block(torch.from_numpy(x).cuda())
    g.reset()
    y = multitone(2000, 4)
    got = g.process_block(torch.from_numpy(y).cuda())[0].cpu().numpy()
    assert np.array_equal(got, oracle.sdm_bits(ref, y))
    g.close()


def test_continuous_blocks_no_gap(oracle):
    """test_continuous_blocks_no_gap: 20 blocks of 64 at lat 64 give
    1,280 - 64 decisions in total, equal to one pass over the same input."""
    g, (ref,) = _pair(oracle, lat=64)
    n = np.arange(1280)
    x = 0.3 * np.sin(2 * np.pi * 1000.0 * n / DSD64)
    got = [g.process_block(torch.from_numpy(x[b * 64:(b + 1) * 64]).cuda())[0].cpu().numpy()
           for b in range(20)]
    got = np.concatenate(got)
    assert len(got) == 1280 - 64
    assert np.array_equal(got, oracle.sdm_bits(ref, x))
    g.close()


def test_reset_one_channel_keeps_the_other(oracle):
    """test_reset_clears_state per channel: resetting context 0 restarts its
    stream and leaves context 1's stream running."""
    g, refs = _pair(oracle, nctx=2)
    xs = np.stack([sdm_input(4000, 21), sdm_input(4000, 22)])
    g.process_block(torch.from_numpy(np.ascontiguousarray(xs[:, :1500])).cuda())
    for c in range(2):
        oracle.sdm_bits(refs[c], xs[c, :1500])
    g.reset(0)
    refs[0].reset()
    got = g.process_block(torch.from_numpy(np.ascontiguousarray(xs[:, 1500:])).cuda())
    for c in range(2):
        want = oracle.sdm_bits(refs[c], xs[c, 1500:])
        assert np.array_equal(got[c].cpu().numpy(), want), c
    g.close()


def test_close_twice_and_destroy_null():
    """test_engine_double_free_safe: closing a wrapper twice is harmless, and
    dsdgpu_destroy(NULL) is a no-op."""
    from foo_dsd_trellis_gb300 import _lib
    from foo_dsd_trellis_gb300.sdm import TrellisSdm
    f = _f()
    g = TrellisSdm(f.order, f.a, f.g, 16, 8, 64)
    g.close()
    g.close()
    _lib.load().dsdgpu_destroy(None)
