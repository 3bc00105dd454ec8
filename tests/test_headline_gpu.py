"""The headline conversion at its own scale, compared with the oracle bit for bit.

DSD128 stereo, 10 s of the 48 kHz multitone + pink signal (seed 1001) through
the whole-path entry point exactly as the benchmark runs it: boxcar 8, the
7-stage FIR chain at the PCM gain with the soft clip, CLANS-7, K = 32,
depth 64, lat 128, 65,536-sample DAS segments (937 per channel, overlap
8,192), full-parallel seeding, DoP output.  The expected bytes are the
oracle's DAS (the trellis pinned to the reference's trellis.c, the seam search
and assembly of src/dsp_plugin.c:2414-2725) run on the GPU's own FIR output,
DoP-packed per channel and interleaved as the plugin writes frames
(src/dop.c:114-136, src/threadpool.c:329-345).

The balanced launch (sdm_parts_kernel: segments cut into 1,024-sample parts,
the context stored and reloaded at every part boundary) and the plain one
segment per warp launch are both compared, and seg0-first seeding (the
reference's rule below DSD512, src/dsp_plugin.c:2185-2283) on a 1.5 s slice.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FS_IN, FS_OUT, NCH = 48000, 6144000, 2
DEPTH, K, LAT, SEG = 64, 32, 128, 65536


def _dop_interleaved(oracle, bits):
    """[nch, n] decisions -> DoP bytes [n/16][nch][3] (phase 0 per channel)."""
    frames = [oracle.dop_pack_bits(bits[c], 0)[0].reshape(-1, 3) for c in range(bits.shape[0])]
    return np.stack(frames, axis=1).reshape(-1)


def _gpu_fir(pcm):
    from foo_dsd_trellis_gb300.fir import FirChain
    from foo_dsd_trellis_gb300.pipeline import PCM_FIR_GAIN
    fc = FirChain(FS_IN, FS_OUT, boxcar_taps=8, soft_clip=True, num_channels=NCH)
    y = fc.process(torch.from_numpy(pcm).cuda(), PCM_FIR_GAIN, PCM_FIR_GAIN).cpu().numpy()
    fc.close()
    return y


def _encode(pcm, seed_mode, balance=None):
    """The whole path on the device; returns (DoP bytes, SDM kernel name)."""
    from foo_dsd_trellis_gb300 import _lib, ntf
    from foo_dsd_trellis_gb300.pipeline import OUT_DOP, Encoder
    f = ntf.get_filter("clans-7", FS_OUT)
    enc = Encoder(FS_IN, FS_OUT, NCH, f, DEPTH, K, LAT, seg_len=SEG, seed_mode=seed_mode,
                  reposition=True, boxcar_taps=8, soft_clip=True, output_format=OUT_DOP)
    if balance is not None:
        _lib.check(enc.h, enc.L.dsdgpu_set_option(enc.h, _lib.OPT_SDM_BALANCE, balance))
    frames = pcm.shape[1]
    out = torch.zeros(enc.out_capacity(frames) + 64, dtype=torch.uint8, device="cuda")
    _, nbytes = enc.process(torch.from_numpy(pcm).cuda(), out)
    kernel = enc.last_sdm_kernel()
    enc.close()
    return out[:nbytes].cpu().numpy(), kernel


def _oracle_dop(oracle, fir, seed_mode):
    from foo_dsd_trellis_gb300 import ntf
    f = ntf.get_filter("clans-7", FS_OUT)
    bits, _, _ = oracle.das_run(f.order, np.array(f.a), np.array(f.g), DEPTH, K, LAT, 0.0, fir,
                                seg_len=SEG, seed_mode=seed_mode, reposition=True,
                                nthreads=os.cpu_count())
    return _dop_interleaved(oracle, bits)


@pytest.fixture(scope="module")
def headline(oracle):
    from foo_dsd_trellis_gb300 import signals
    pcm = signals.dsd128_multitone_pink(10.0, FS_IN, NCH, 1001)
    want = _oracle_dop(oracle, _gpu_fir(pcm), 0)
    return pcm, want


@pytest.mark.parametrize("balance,kernel", [(None, "sdm_parts_kernel<7>"),
                                            (0, "sdm_jobs_kernel<7,32>")],
                         ids=["balanced_auto", "one_segment_per_warp"])
def test_headline_10s_bit_exact(headline, balance, kernel):
    pcm, want = headline
    got, ran = _encode(pcm, 0, balance)
    assert ran == kernel
    # 10 s at 6.144 MHz minus the full-parallel seg0 cut (one overlap), both channels
    assert len(want) == (FS_OUT * 10 - 64 * LAT) // 16 * 3 * NCH
    assert len(got) == len(want)
    bad = np.nonzero(got != want)[0]
    assert bad.size == 0, f"{bad.size} DoP bytes differ, first at byte {bad[:4]}"


def test_headline_seg0_first_bit_exact(oracle):
    """seg0-first seeding (seg0 serial, seg1 from its final state, seg2+ from
    the 16-level estimate) on the first 1.5 s of the same signal."""
    from foo_dsd_trellis_gb300 import signals
    pcm = np.ascontiguousarray(signals.dsd128_multitone_pink(10.0, FS_IN, NCH, 1001)[:, :72000])
    want = _oracle_dop(oracle, _gpu_fir(pcm), 1)
    got, _ = _encode(pcm, 1)
    assert len(got) == len(want)
    assert np.array_equal(got, want)
