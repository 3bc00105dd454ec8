"""The differentiable path: exact forward decisions, the hand-written adjoint
against PyTorch autograd of the same surrogate, and against FP64 central
finite differences (h = 1e-6) of the surrogate with the decisions frozen,
on random parameter directions (relative agreement 1e-4)."""
import numpy as np
import pytest

from signals import multitone, uniform_noise

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _clips(nclips, frames, fs, seed):
    out = np.empty((nclips, frames), np.float32)
    for c in range(nclips):
        x = 0.25 * multitone(frames, 5 + c + seed) + uniform_noise(frames, 40 + c + seed, 1e-3)
        out[c] = x.astype(np.float32)
    return out


def _engine(cfg, order_name="clans-7"):
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.diff import DiffEngine
    f = ntf.get_filter(order_name, cfg.fs_out)
    return DiffEngine(cfg, f), f


def _params(cfg, f, seed=3):
    rng = np.random.default_rng(seed)
    taps = rng.normal(0.0, 1e-3, cfg.preemph_taps)
    taps[0] += 1.0
    return taps, np.array(f.a[: f.order]), np.array(f.g[: f.order])


def test_forward_decisions_are_the_exact_trellis(oracle):
    from foo_dsd_trellis_gb300.diff import DiffConfig
    cfg = DiffConfig(fs_in=44100, fs_out=5644800, nclips=3, frames=512, cands=16, depth=32,
                     lat=32, checkpoint=4096)
    eng, f = _engine(cfg)
    eng.set_input(torch.from_numpy(_clips(3, 512, 44100, 0)).cuda())
    taps, a, g = _params(cfg, f)
    loss = eng.forward(taps, a, g)
    assert np.isfinite(loss) and loss > 0
    u, bits = eng.buffers()
    u, bits = u.cpu().numpy(), bits.cpu().numpy()
    for c in range(3):
        ctx = oracle.sdm(f.order, np.array(f.a), np.array(f.g), 32, 16, 32)
        want = oracle.sdm_bits(ctx, np.concatenate([u[c], np.zeros(32)]))
        assert np.array_equal(bits[c], want), f"clip {c}"
    eng.close()


def test_adjoint_matches_autograd(oracle):
    import diff_reference as R
    from foo_dsd_trellis_gb300.diff import DiffConfig
    cfg = DiffConfig(fs_in=1411200, fs_out=5644800, nclips=2, frames=1024, preemph_taps=15,
                     decim=16, lpf_taps=63, lpf_cutoff_hz=100000.0, cands=8, depth=16, lat=16,
                     checkpoint=256, gain=0.5)
    eng, f = _engine(cfg)
    x = _clips(2, 1024, 1411200, 1)
    eng.set_input(torch.from_numpy(x).cuda())
    taps, a, g = _params(cfg, f)
    loss = eng.forward(taps, a, g)
    gt, ga, gg = eng.backward()
    _, bits = eng.buffers()
    ybits = torch.from_numpy(bits.cpu().numpy().astype(np.float64) * 2.0 - 1.0)
    xt = torch.from_numpy(x.astype(np.float64))
    h = torch.from_numpy(R.lpf_taps(cfg.lpf_taps, cfg.lpf_cutoff_hz, cfg.fs_out))
    r = R.chain(oracle, cfg.fs_in, cfg.fs_out, xt, cfg.gain)
    T = torch.tensor(taps, requires_grad=True)
    A = torch.tensor(a, requires_grad=True)
    G = torch.tensor(g, requires_grad=True)
    with torch.no_grad():
        u0 = R.chain(oracle, cfg.fs_in, cfg.fs_out, R._causal(xt, T), cfg.gain)
        beta = R.base_beta(u0, ybits, A, G, cfg.kappa)
        want_loss = R.loss_of(ybits, r, h, cfg.decim)
    assert loss == pytest.approx(float(want_loss), rel=1e-9)
    L = R.surrogate(oracle, cfg, xt, T, A, G, beta, r, h)
    assert float(L.detach()) == pytest.approx(float(want_loss), rel=1e-8)
    L.backward()
    np.testing.assert_allclose(gt, T.grad.numpy(), rtol=1e-6, atol=1e-9 * np.abs(gt).max())
    np.testing.assert_allclose(ga, A.grad.numpy(), rtol=1e-6, atol=1e-9 * np.abs(ga).max())
    np.testing.assert_allclose(gg, G.grad.numpy(), rtol=1e-6, atol=1e-9 * np.abs(gg).max())
    eng.close()


@pytest.mark.parametrize("ndir", [32])
def test_adjoint_matches_finite_differences(ndir):
    """Central differences (h = 1e-6, FP64) of the surrogate, decisions frozen,
    on random directions over (taps, a, g): 1e-4 relative.  Every gradient
    component, the zero g entries included, is checked against autograd above."""
    from foo_dsd_trellis_gb300.diff import DiffConfig
    cfg = DiffConfig(fs_in=44100, fs_out=5644800, nclips=4, frames=1024, cands=8, depth=16,
                     lat=16, checkpoint=4096)
    eng, f = _engine(cfg)
    eng.set_input(torch.from_numpy(_clips(4, 1024, 44100, 2)).cuda())
    taps, a, g = _params(cfg, f)
    L0 = eng.forward(taps, a, g)
    gt, ga, gg = eng.backward()
    assert eng.surrogate(taps, a, g) == pytest.approx(L0, rel=1e-9)
    rng = np.random.default_rng(11)
    h = 1e-6
    worst = 0.0
    for k in range(ndir):
        # a random direction: absolute for the taps, relative for the NTF
        # coefficients (a_i n_i, g_i n_i; structural zeros of g stay zero --
        # an absolute step in a or g of 1e-6 moves the loop states, which
        # reach ~1e5, far outside the linear regime)
        dt = rng.standard_normal(taps.size)
        da = a * rng.standard_normal(a.size)
        dg = g * rng.standard_normal(g.size)
        lp = eng.surrogate(taps + h * dt, a + h * da, g + h * dg)
        lm = eng.surrogate(taps - h * dt, a - h * da, g - h * dg)
        fd = (lp - lm) / (2 * h)
        ad = gt @ dt + ga @ da + gg @ dg
        rel = abs(fd - ad) / max(abs(fd), abs(ad), 1e-300)
        worst = max(worst, rel)
        assert rel < 1e-4, f"direction {k}: fd {fd} adjoint {ad} rel {rel}"
    eng.close()


def test_autograd_function_and_training_step():
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.diff import DiffConfig, SdmLoss
    cfg = DiffConfig(fs_in=44100, fs_out=5644800, nclips=2, frames=512, cands=8, depth=16,
                     lat=16, checkpoint=4096)
    f = ntf.get_filter("clans-7", cfg.fs_out)
    m = SdmLoss(cfg, f)
    m.set_input(torch.from_numpy(_clips(2, 512, 44100, 4)).cuda())
    loss = m()
    loss.backward()
    assert m.taps.grad is not None and m.taps.grad.dtype == torch.float32
    assert torch.isfinite(m.a.grad).all() and torch.isfinite(m.g.grad).all()
    gt, ga, gg = m.engine.backward()
    np.testing.assert_allclose(m.a.grad.numpy(), ga, rtol=1e-12)
    opt = torch.optim.SGD(m.parameters(), lr=1e-3)
    opt.step()
    assert torch.isfinite(m().detach())
