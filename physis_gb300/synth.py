"""Seeded synthetic inputs shared by the benchmarks and the tests.

uniform(shape, seed): float32 in [0,1) from a counter-based SplitMix64
stream (Steele, Lea and Flood, "Fast splittable pseudorandom number
generators", OOPSLA 2014): element i is (splitmix64(seed*2^32 + i) >> 40)
* 2^-24, i.e. 24 random bits, in x-fastest (C) order of `shape` = (nz,ny,nx).
"""
import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _splitmix64(z):
    z = z + _GOLDEN
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def uniform(shape, seed, out=None, chunk=1 << 24):
    n = int(np.prod(shape))
    if out is None:
        out = np.empty(shape, dtype=np.float32)
    flat = out.reshape(-1)
    base = np.uint64(int(seed) << 32)
    scale = np.float32(1.0 / 16777216.0)
    with np.errstate(over="ignore"):
        for s in range(0, n, chunk):
            e = min(n, s + chunk)
            idx = np.arange(s, e, dtype=np.uint64) + base
            r = _splitmix64(idx) >> np.uint64(40)
            flat[s:e] = r.astype(np.float32) * scale
    return out
