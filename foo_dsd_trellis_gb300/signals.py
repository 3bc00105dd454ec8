"""Seeded synthetic PCM signals with the shapes of the conversion workloads:
multitone (log-spaced tones at a fixed level with random phases), pink noise
at a fixed RMS, a sine with TPDF dither, band-limited Gaussian noise.  The
generator is numpy's PCG64 with seed 1000 + workload index, offset by the
channel index."""
from __future__ import annotations

import numpy as np


def db_to_amp(db: float) -> float:
    return float(10.0 ** (db / 20.0))


def pink_noise(n: int, rng: np.random.Generator, rms: float) -> np.ndarray:
    """White Gaussian noise shaped to a 1/f power spectrum in the FFT domain."""
    w = rng.standard_normal(n)
    spec = np.fft.rfft(w)
    f = np.arange(len(spec), dtype=np.float64)
    f[0] = 1.0
    spec /= np.sqrt(f)
    spec[0] = 0.0
    x = np.fft.irfft(spec, n)
    return x * (rms / np.sqrt(np.mean(x * x)))


def multitone(n: int, fs: float, rng: np.random.Generator, ntones: int = 31, f_lo: float = 20.0,
              f_hi: float = 20000.0, level_db: float = -20.0) -> np.ndarray:
    freqs = np.geomspace(f_lo, f_hi, ntones)
    ph = rng.random(ntones) * 2 * np.pi
    t = np.arange(n) / fs
    amp = db_to_amp(level_db)
    x = np.zeros(n)
    for f, p in zip(freqs, ph):
        x += amp * np.sin(2 * np.pi * f * t + p)
    return x


def dsd128_multitone_pink(seconds: float, fs: int = 48000, channels: int = 2,
                          seed: int = 1001) -> np.ndarray:
    """31 log-spaced tones 20 Hz-20 kHz at -20 dBFS each with random phases plus
    pink noise at -30 dBFS: the DSD128 DAS workload's input, float32 [ch, n]."""
    n = int(round(seconds * fs))
    out = np.empty((channels, n), np.float32)
    for c in range(channels):
        rng = np.random.Generator(np.random.PCG64(seed + c))
        out[c] = (multitone(n, fs, rng) + pink_noise(n, rng, db_to_amp(-30.0))).astype(np.float32)
    return out


def sine_tpdf(seconds: float, fs: int = 44100, channels: int = 2, f0: float = 997.0,
              level_db: float = -6.0, dither_db: float = -110.0, seed: int = 1000) -> np.ndarray:
    """A sine at level_db plus TPDF dither at dither_db RMS, float32 [ch, n]."""
    n = int(round(seconds * fs))
    t = np.arange(n) / fs
    out = np.empty((channels, n), np.float32)
    for c in range(channels):
        rng = np.random.Generator(np.random.PCG64(seed + c))
        tpdf = rng.random(n) - rng.random(n)                  # RMS 1/sqrt(6)
        d = tpdf * db_to_amp(dither_db) * np.sqrt(6.0)
        out[c] = (db_to_amp(level_db) * np.sin(2 * np.pi * f0 * t) + d).astype(np.float32)
    return out


def bandlimited_noise(n: int, fs: int, rng: np.random.Generator, rms: float,
                      f_hi: float = 20000.0) -> np.ndarray:
    """White Gaussian noise low-passed at f_hi (FFT-domain brick wall), scaled
    to `rms`."""
    w = rng.standard_normal(n)
    spec = np.fft.rfft(w)
    f = np.fft.rfftfreq(n, 1.0 / fs)
    spec[f > f_hi] = 0.0
    x = np.fft.irfft(spec, n)
    return x * (rms / max(1e-30, float(np.sqrt(np.mean(x * x)))))


# DSD targets of the 44.1 kHz and 48 kHz families
_FAMILY = {44100: (5644800, 11289600), 88200: (5644800, 11289600), 176400: (5644800, 11289600),
           48000: (6144000, 12288000), 96000: (6144000, 12288000), 192000: (6144000, 12288000)}


def multistream_layout(nstreams: int = 64, seed: int = 1003, len_lo: float = 0.5,
                       len_hi: float = 30.0, scale: float = 1.0) -> list[dict]:
    """The batched workload's stream table: lengths U(len_lo, len_hi) s (times
    `scale`), input rates drawn from {44.1, 48, 88.2, 96, 176.4, 192} kHz,
    targets DSD128 or DSD256 of the matching family, stereo."""
    rng = np.random.Generator(np.random.PCG64(seed))
    rates = sorted(_FAMILY)
    out = []
    for i in range(nstreams):
        fs = int(rates[rng.integers(len(rates))])
        fo = int(_FAMILY[fs][rng.integers(2)])
        sec = float(rng.uniform(len_lo, len_hi)) * scale
        out.append({"fs_in": fs, "fs_out": fo, "channels": 2,
                    "frames": max(1, int(round(sec * fs))), "seed": seed * 1000 + i})
    return out


def multistream_pcm(entry: dict, level_db: float = -12.0) -> np.ndarray:
    """One stream of the batched workload: band-limited Gaussian noise at
    level_db RMS, float32 [channels, frames]."""
    n, ch = entry["frames"], entry["channels"]
    out = np.empty((ch, n), np.float32)
    for c in range(ch):
        rng = np.random.Generator(np.random.PCG64(entry["seed"] + c))
        out[c] = bandlimited_noise(n, entry["fs_in"], rng, db_to_amp(level_db)).astype(np.float32)
    return out


def dop_floats(bits01: np.ndarray, phase: int = 0) -> np.ndarray:
    """0/1 decision bytes [n] -> DoP float samples (the 24-bit frame
    [marker, 16 decisions MSB first] as a signed value / 2^23), markers
    alternating 0x05 / 0xFA from `phase`: what a decoder hands the plugin."""
    bits01 = np.asarray(bits01, np.uint8)
    frames = len(bits01) // 16
    b = np.packbits(bits01[: 16 * frames].reshape(frames, 16), axis=1).astype(np.int32)
    w = (b[:, 0] << 8) | b[:, 1]
    marker = np.where((np.arange(frames) + phase) % 2 == 0, 0x05, 0xFA).astype(np.int32)
    v = (marker << 16) | w
    v = np.where(v >= 1 << 23, v - (1 << 24), v)
    return (v.astype(np.float64) / 8388608.0).astype(np.float32)
