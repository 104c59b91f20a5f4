"""Seeded synthetic inputs for the five benchmark workloads.

No public dataset is involved: every input is synthetic, drawn from the
distribution each workload specifies.  numpy's PCG64 generator is
platform-independent, so the same seed gives the same input on any host.
The torch variants generate the large workloads directly in device memory
(same distributions, torch's own generator; reproducible per seed on a given
torch build, not bit-equal to the numpy variant).
"""
from __future__ import annotations

import numpy as np

# ---------------------------------------------------------------- workload 1
# Complex forward then inverse round trip: N = 1024 complex FP32 interleaved,
# 4096 independent transforms, re/im i.i.d. uniform[-1, 1), seed 0.
W1_N, W1_FRAMES, W1_SEED = 1024, 4096, 0


def complex_uniform(frames: int, n: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    re = rng.uniform(-1.0, 1.0, size=(frames, n))
    im = rng.uniform(-1.0, 1.0, size=(frames, n))
    return (re + 1j * im).astype(np.complex64)


# ---------------------------------------------------------------- workload 2
# Real forward / inverse: N = 4096 real FP32, 65536 frames.  Each frame is a
# sum of 8 sinusoids (frequency uniform in (0, N/2) bins, amplitude uniform
# [0.1, 1], phase uniform [0, 2 pi)) plus Gaussian noise sigma = 0.01.
W2_N, W2_FRAMES, W2_SEED = 4096, 65536, 2
W2_TONES, W2_NOISE = 8, 0.01


def sine_frames(frames: int, n: int, seed: int = W2_SEED, tones: int = W2_TONES,
                noise: float = W2_NOISE) -> np.ndarray:
    rng = np.random.default_rng(seed)
    f = rng.uniform(0.0, n / 2, size=(frames, tones, 1))
    a = rng.uniform(0.1, 1.0, size=(frames, tones, 1))
    ph = rng.uniform(0.0, 2 * np.pi, size=(frames, tones, 1))
    t = np.arange(n)[None, None, :]
    x = (a * np.cos(2 * np.pi * f * t / n + ph)).sum(axis=1)
    x += rng.normal(0.0, noise, size=(frames, n))
    return x.astype(np.float32)


def sine_frames_torch(frames: int, n: int, seed: int = W2_SEED, device="cuda",
                      tones: int = W2_TONES, noise: float = W2_NOISE, chunk: int = 8192):
    """Same distribution generated on the device in chunks (float32 output)."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    out = torch.empty((frames, n), dtype=torch.float32, device=device)
    t = torch.arange(n, device=device, dtype=torch.float64)[None, None, :]
    for s in range(0, frames, chunk):
        c = min(chunk, frames - s)
        f = torch.rand((c, tones, 1), generator=g, device=device, dtype=torch.float64) * (n / 2)
        a = 0.1 + 0.9 * torch.rand((c, tones, 1), generator=g, device=device, dtype=torch.float64)
        ph = 2 * np.pi * torch.rand((c, tones, 1), generator=g, device=device, dtype=torch.float64)
        x = (a * torch.cos(2 * np.pi * f * t / n + ph)).sum(dim=1)
        x += noise * torch.randn((c, n), generator=g, device=device, dtype=torch.float64)
        out[s:s + c] = x.to(torch.float32)
    return out


# ---------------------------------------------------------------- workload 3
# Large single transforms: complex N = 2^20, 2^22, 2^24, re/im i.i.d. N(0, 1).
W3_LOG2 = (20, 22, 24)


def complex_normal(n: int, seed: int = 3) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)


# ---------------------------------------------------------------- workload 4
# Uneven batch: 10000 transforms, log2 N uniform in {6..16}, 70% complex /
# 30% real, 50% forward / 50% inverse, inputs i.i.d. uniform[-1, 1).
W4_JOBS, W4_LOG2, W4_SEED = 10000, (6, 16), 4


def uneven_jobs(count: int = W4_JOBS, seed: int = W4_SEED, log2_range=W4_LOG2):
    """List of (real: bool, inverse: bool, log2n: int)."""
    rng = np.random.default_rng(seed)
    lo, hi = log2_range
    l2 = rng.integers(lo, hi + 1, size=count)
    real = rng.uniform(size=count) < 0.3
    inv = rng.uniform(size=count) < 0.5
    return [(bool(r), bool(i), int(l)) for r, i, l in zip(real, inv, l2)]


# ---------------------------------------------------------------- workload 5
# Serving: Poisson arrivals; each request has size 2^k, k uniform in {8..20},
# 1-64 frames, mixed complex/real, inputs i.i.d. N(0, 1).
W5_LOG2, W5_SEED = (8, 20), 5


def serving_requests(count: int, rate_per_s: float, seed: int = W5_SEED, log2_range=W5_LOG2,
                     max_frames: int = 64):
    """List of (arrival_s, real, inverse, log2n, frames)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, size=count)
    t = np.cumsum(gaps) - gaps[0]
    lo, hi = log2_range
    l2 = rng.integers(lo, hi + 1, size=count)
    frames = rng.integers(1, max_frames + 1, size=count)
    real = rng.uniform(size=count) < 0.5
    inv = rng.uniform(size=count) < 0.5
    return [(float(a), bool(r), bool(i), int(l), int(f)) for a, r, i, l, f in zip(t, real, inv, l2, frames)]


# ------------------------------------------------------------------ bytes
def algorithmic_bytes(real: bool, n: int) -> int:
    """HBM bytes one transform must move at minimum (read input once, write output once):
    complex 16 n; real 4 n + 8 (n/2 + 1) in either direction."""
    return 4 * n + 8 * (n // 2 + 1) if real else 16 * n
