"""GPU DoP / native packers vs the oracle restatement of src/dop.c (bit-exact)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("n", [0, 15, 16, 17, 1000, 65536 + 9])
@pytest.mark.parametrize("phase", [0, 1])
def test_dop_and_native(oracle, n, phase):
    from foo_dsd_trellis_gb300.pack import Packer
    rng = np.random.default_rng(n + phase)
    bits = (rng.random((3, n)) > 0.5).astype(np.uint8)
    p = Packer()
    dop, ph = p.dop(torch.from_numpy(bits).cuda(), phase)
    dop = dop.cpu().numpy()
    nat = p.native(torch.from_numpy(bits).cuda()).cpu().numpy()
    for c in range(3):
        want, wph = oracle.dop_pack_bits(bits[c], phase)
        assert wph == ph
        assert np.array_equal(dop[:, c, :].reshape(-1), want)
        assert np.array_equal(nat[c], oracle.bits_pack(bits[c]))


def test_dop_unpack_pack_roundtrip(oracle):
    """DoP frames unpacked on the GPU and packed again give the same 24-bit
    frames (the reference's round trip, test/test_hardening.c:613-647): the
    decisions in the low 16 bits and the marker byte alternating from the
    phase."""
    import ctypes as C
    from foo_dsd_trellis_gb300 import _lib
    from foo_dsd_trellis_gb300.pack import Packer
    rng = np.random.default_rng(12)
    frames, nch = 4099, 2
    bits = (rng.random((nch, 16 * frames)) > 0.5).astype(np.uint8)
    dop = np.stack([oracle.dop_float_frames(bits[c], 1) for c in range(nch)])
    L = _lib.load()
    h = C.c_void_p()
    assert L.dsdgpu_create(0, C.byref(h)) == 0
    d_dop = torch.from_numpy(dop).cuda()
    un = torch.empty((nch, 16 * frames), dtype=torch.uint8, device="cuda")
    _lib.check(h, L.dsdgpu_dop_unpack(h, nch, C.c_void_p(d_dop.data_ptr()), frames, frames,
                                      C.c_void_p(un.data_ptr()), 16 * frames))
    torch.cuda.synchronize()
    L.dsdgpu_destroy(h)
    assert np.array_equal(un.cpu().numpy(), bits)
    p = Packer()
    packed, ph = p.dop(un, 1)
    packed = packed.cpu().numpy()
    for c in range(nch):
        want, wph = oracle.dop_pack_bits(bits[c], 1)
        assert wph == ph
        assert np.array_equal(packed[:, c, :].reshape(-1), want)
        # the float frames encode the same 24-bit words
        words = np.round(dop[c].astype(np.float64) * 8388608.0).astype(np.int64) & 0xFFFFFF
        got = (packed[:, c, 0].astype(np.int64) | (packed[:, c, 1].astype(np.int64) << 8)
               | (packed[:, c, 2].astype(np.int64) << 16))
        assert np.array_equal(got, words)
