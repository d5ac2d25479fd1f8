"""Synthetic workload definitions (seeded initial fields, equation strings).

Initial fields come from a seeded SplitMix64 stream mapped to uniform floats, so
the same field can be regenerated bit-for-bit anywhere (seed 20261203 by default).
"""
from __future__ import annotations

import numpy as np

DEFAULT_SEED = 20261203


def splitmix64_uniform(n, seed=DEFAULT_SEED, lo=-0.1, hi=0.1):
    """n float32 values uniform in [lo, hi) from SplitMix64 (Steele, Lea, Flood 2014)."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(40)).astype(np.float64) * 2.0 ** -24
    return (lo + (hi - lo) * u).astype(np.float32)


# Equation strings in reference syntax (cf. examples/02_cahn_hilliard, 03_cahn_hilliard_3d,
# 05_edwards_wilkinson, 06_kpz of the reference).
CH_EQ = "dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"
CH_NOISE = "2*T*q^2"
