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
