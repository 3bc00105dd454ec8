"""PyTorch FP64 reference of the differentiable path's loss and surrogate,
used by the tests to check the hand-written adjoint against autograd.

Chain taps come from the oracle's restatement of the reference's half-band
design (src/fir.c:65-150); the NTF loop follows src/trellis.c:104-118 (the
same recurrence, written with tensor ops so autograd differentiates it)."""
import math

import numpy as np
import torch


def lpf_taps(T: int, cutoff_hz: float, fs: float) -> np.ndarray:
    """Kaiser (beta 10) windowed sinc, unit DC gain."""
    fc = cutoff_hz / fs

    def i0(x):
        s = t = 1.0
        for k in range(1, 60):
            t *= (x / (2.0 * k)) ** 2
            s += t
        return s

    h = np.zeros(T)
    for k in range(T):
        m = k - (T - 1) / 2.0
        sinc = 2.0 * fc if m == 0 else math.sin(2 * math.pi * fc * m) / (math.pi * m)
        q = 2.0 * k / (T - 1) - 1.0 if T > 1 else 0.0
        w = i0(10.0 * math.sqrt(max(0.0, 1.0 - q * q))) / i0(10.0) if T > 1 else 1.0
        h[k] = sinc * w
    return h / h.sum()


def _causal(x: torch.Tensor, h: torch.Tensor) -> torch.Tensor:
    """y[c, m] = sum_k h[k] x[c, m - k] (zero history)."""
    T = h.numel()
    xp = torch.nn.functional.pad(x, (T - 1, 0))
    return torch.nn.functional.conv1d(xp.unsqueeze(1), h.flip(0).view(1, 1, -1)).squeeze(1)


def chain(oracle, fs_in, fs_out, x: torch.Tensor, gain: float) -> torch.Tensor:
    for U, L in oracle.fir_plan(fs_in, fs_out):
        h = torch.from_numpy(oracle.fir_design(L, U == 4) * U)
        zs = torch.zeros(x.shape[0], x.shape[1] * U, dtype=torch.float64)
        zs[:, ::U] = x
        x = _causal(zs, h)
    return x * gain


def loss_of(y: torch.Tensor, r: torch.Tensor, h: torch.Tensor, D: int) -> torch.Tensor:
    e = (y - r).unsqueeze(1)
    z = torch.nn.functional.conv1d(e, h.view(1, 1, -1)).squeeze(1)[:, ::D]
    return (z * z).mean()


def base_beta(u, ybits, a, g, kappa):
    """beta_t = y^_t - kappa v^_t along the loop driven by the decisions."""
    C, n = u.shape
    N = a.numel()
    s = torch.zeros(C, N, dtype=torch.float64)
    beta = torch.empty(C, n, dtype=torch.float64)
    for t in range(n):
        d = _loop_d(s, u[:, t], g)
        v = u[:, t] + (a * d).sum(1)
        beta[:, t] = ybits[:, t] - kappa * v
        s = torch.cat([(d[:, 0] - ybits[:, t]).unsqueeze(1), d[:, 1:]], 1)
    return beta


def _loop_d(s, x, g):
    N = s.shape[1]
    cols = [s[:, 0] - g[0] * s[:, 1] + x]
    for i in range(1, N - 1):
        cols.append(s[:, i] + s[:, i - 1] - g[i] * s[:, i + 1])
    cols.append(s[:, N - 1] + s[:, N - 2])
    return torch.stack(cols, 1)


def surrogate(oracle, cfg, x, taps, a, g, beta, r, h):
    """The straight-through surrogate: y = kappa v + beta with the loop driven by y."""
    p = _causal(x, taps)
    u = chain(oracle, cfg.fs_in, cfg.fs_out, p, cfg.gain)
    C, n = u.shape
    N = a.numel()
    s = torch.zeros(C, N, dtype=torch.float64)
    ys = []
    for t in range(n):
        d = _loop_d(s, u[:, t], g)
        v = u[:, t] + (a * d).sum(1)
        y = cfg.kappa * v + beta[:, t]
        s = torch.cat([(d[:, 0] - y).unsqueeze(1), d[:, 1:]], 1)
        ys.append(y)
    return loss_of(torch.stack(ys, 1), r, h, cfg.decim)
