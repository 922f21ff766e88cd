"""Host restatement of the device's seeded uniform generator (nt2cuda_fill_uniform_f32/f64).

The device fills element i of a table from a counter-based hash of (seed, i):
h = splitmix64(seed * 0xd1342543de82ef95 + splitmix64(i)), then
u = top 24 bits / 2^24 (float) or top 53 bits / 2^53 (double) and
x = lo + (hi - lo) * u, each operation rounded once.  The same arithmetic in
numpy gives the same tables on the host bit for bit, so CPU runs (the CPU
baseline, the tests) can use the GPU's inputs without reading them back.
"""
from __future__ import annotations

import numpy as np

_M = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    x = x + np.uint64(0x9E3779B97F4A7C15)
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def _hash2(seed: int, i: np.ndarray) -> np.ndarray:
    s = np.uint64((seed * 0xD1342543DE82EF95) & 0xFFFFFFFFFFFFFFFF)
    return _splitmix64(s + _splitmix64(i))


def uniform_f32(n: int, lo: float, hi: float, seed: int, chunk: int = 1 << 22) -> np.ndarray:
    """The table nt2cuda_fill_uniform_f32(x, n, lo, hi, seed) writes."""
    out = np.empty(n, np.float32)
    lo32, hi32 = np.float32(lo), np.float32(hi)
    w = np.float32(hi32 - lo32)
    with np.errstate(over="ignore"):
        for a in range(0, n, chunk):
            i = np.arange(a, min(n, a + chunk), dtype=np.uint64)
            u = (_hash2(seed, i) >> np.uint64(40)).astype(np.float32) * np.float32(1.0 / 16777216.0)
            out[a:a + i.size] = lo32 + w * u
    return out


def uniform_f64(n: int, lo: float, hi: float, seed: int, chunk: int = 1 << 22) -> np.ndarray:
    """The table nt2cuda_fill_uniform_f64(x, n, lo, hi, seed) writes."""
    out = np.empty(n, np.float64)
    w = np.float64(hi) - np.float64(lo)
    with np.errstate(over="ignore"):
        for a in range(0, n, chunk):
            i = np.arange(a, min(n, a + chunk), dtype=np.uint64)
            u = (_hash2(seed, i) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
            out[a:a + i.size] = np.float64(lo) + w * u
    return out


def blackscholes_inputs(n: int, seed: int, dtype=np.float32):
    """S ~ U[5,30], K ~ U[1,100], T ~ U[0.25,10] as the benchmark fills them on the device
    (seeds 3*seed+1, 3*seed+2, 3*seed+3)."""
    f = uniform_f32 if dtype == np.float32 else uniform_f64
    return (f(n, 5.0, 30.0, 3 * seed + 1), f(n, 1.0, 100.0, 3 * seed + 2), f(n, 0.25, 10.0, 3 * seed + 3))
