"""Seeded, platform-independent test signals for the SDM parity tests.

Only IEEE add/multiply and numpy's PCG64 uniform doubles are used, so the same
seed gives bit-identical inputs on x86_64 and aarch64 (no libm calls whose last
ulp could differ between machines).
"""
from __future__ import annotations

import numpy as np


def rotation_sine(n: int, cycles_per_sample: float, amp: float) -> np.ndarray:
    """amp * sin(2 pi f t) by a complex-rotation recurrence.  The rotation
    constant is computed with numpy once and rounded to a fixed number of
    significant bits so that it is identical everywhere."""
    th = 2.0 * np.pi * cycles_per_sample
    c = float(np.float64(np.round(np.cos(th) * 2**40) / 2**40))
    s = float(np.float64(np.round(np.sin(th) * 2**40) / 2**40))
    out = np.empty(n, np.float64)
    re, im = 1.0, 0.0
    for i in range(n):
        out[i] = im
        re, im = re * c - im * s, re * s + im * c
    return amp * out


def uniform_noise(n: int, seed: int, amp: float) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    return amp * (rng.random(n) - rng.random(n))   # triangular (TPDF) shape


def sdm_input(n: int, seed: int, amp: float = 0.5, f: float = 0.0013,
              noise: float = 0.05) -> np.ndarray:
    """A tone plus triangular noise, the shape of the reference's own SDM tests
    (a sine at half scale, test/test_trellis.c:186-207)."""
    return rotation_sine(n, f, amp) + uniform_noise(n, seed, noise)


def multitone(n: int, seed: int, ntones: int = 7, amp: float = 0.08) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    freqs = rng.random(ntones) * 0.004 + 0.0002
    x = np.zeros(n)
    for f in freqs:
        x += rotation_sine(n, float(f), amp)
    return x + uniform_noise(n, seed + 1, 0.02)
