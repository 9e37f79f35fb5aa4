"""Seeded synthetic columns of the benchmark shapes (they stand in for the
reference's UCR2018 / TPC-H / embedding datasets, which are not available).

Values are rounded half away from zero, as Rust's f64::round does, and -0.0 is
normalised to +0.0 so min/max never meet a signed-zero tie.
"""
from __future__ import annotations

import numpy as np


def round_dp(x, dp: int):
    """(x * 10^dp).round() / 10^dp with Rust's half-away-from-zero rounding."""
    s = 10.0 ** dp
    y = np.asarray(x, dtype=np.float64) * s
    r = np.trunc(y)
    r += np.where(np.abs(y - r) >= 0.5, np.sign(y), 0.0)
    return r / s + 0.0


def gorilla_walk(n=1_048_576, seed=1, x0=30.0):
    """x[i] = x[i-1] + N(0, 0.5), rounded to 2 decimals (8,192-value Gorilla chunks)."""
    rng = np.random.default_rng(seed)
    return round_dp(x0 + np.cumsum(rng.normal(0.0, 0.5, n)), 2)


def buff_uniform(n=67_108_864, seed=2):
    """Uniform on [-1000, 1000] rounded to 3 decimals (65,536-value BUFF chunks, scale 1000)."""
    rng = np.random.default_rng(seed)
    out = np.empty(n, dtype=np.float64)
    step = 1 << 24
    for i in range(0, n, step):  # bounded temporaries
        m = min(step, n - i)
        out[i:i + m] = round_dp(rng.uniform(-1000.0, 1000.0, m), 3)
    return out


def sensor(n=16_777_216, seed=3):
    """20 + 10 sin(2 pi i / 1440) + N(0, 0.1), rounded to 4 decimals (Chimp128)."""
    rng = np.random.default_rng(seed)
    i = np.arange(n, dtype=np.float64)
    return round_dp(20.0 + 10.0 * np.sin(2.0 * np.pi * i / 1440.0) + rng.normal(0.0, 0.1, n), 4)


def steps(n=16_777_216, seed=4):
    """Runs of Geometric(1/64) length; levels move by U{-5..5} * 0.1 (RLE)."""
    rng = np.random.default_rng(seed)
    lens = rng.geometric(1.0 / 64.0, n // 32 + 16)
    while lens.sum() < n:
        lens = np.concatenate([lens, rng.geometric(1.0 / 64.0, n // 32 + 16)])
    deltas = rng.integers(-5, 6, len(lens)) * 0.1
    levels = round_dp(50.0 + np.cumsum(deltas), 1)
    return np.repeat(levels, lens)[:n].copy()


# BUFF selectivities of the fused filter+sum bench queries: [-a, a] keeps a / 1000.
BUFF_RANGES = {"1%": 10.0, "10%": 100.0, "50%": 500.0}
