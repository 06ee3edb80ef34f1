"""Seeded synthetic vertex configurations, drawn as the reference draws them.

sample_uniform_unit_vertex (mcmcmc_sampler.h:187-190) takes four
std::uniform_real_distribution<double>(0, 1) draws from a std::mt19937_64;
seeds derive from a base seed with derive_mcmcmc_seed (:159-172). This module
restates both in vectorised numpy (the 64-bit Mersenne Twister of the C++
standard, libstdc++'s generate_canonical for one 64-bit word), so that the
same seed gives the same configurations as the reference sampler.
"""
from __future__ import annotations

import numpy as np

_MASK = (1 << 64) - 1
_N, _M = 312, 156
_UPPER = np.uint64(0xFFFFFFFF80000000)
_LOWER = np.uint64(0x7FFFFFFF)
_MATRIX_A = np.uint64(0xB5026F5AA96619E9)


class MT19937_64:
    """std::mt19937_64 with a vectorised state twist."""

    def __init__(self, seed: int):
        mt = [seed & _MASK]
        for i in range(1, _N):
            prev = mt[-1]
            mt.append((6364136223846793005 * (prev ^ (prev >> 62)) + i) & _MASK)
        self.mt = np.array(mt, dtype=np.uint64)
        self.index = _N

    def _twist(self) -> None:
        mt = self.mt
        one = np.uint64(1)

        def mix(lo, hi_src, far):
            y = (mt[lo] & _UPPER) | (hi_src & _LOWER)
            return far ^ (y >> one) ^ np.where((y & one) != 0, _MATRIX_A, np.uint64(0))

        # i in [0, 156): neighbours i+1 and i+156 are still old
        i = np.arange(0, _N - _M)
        mt[i] = mix(i, mt[i + 1], mt[i + _M])
        # i in [156, 311): i+156-312 = i-156 already new
        i = np.arange(_N - _M, _N - 1)
        mt[i] = mix(i, mt[i + 1], mt[i - (_N - _M)])
        # i = 311 wraps to mt[0] (new)
        y = (mt[_N - 1] & _UPPER) | (mt[0] & _LOWER)
        mt[_N - 1] = mt[_M - 1] ^ (y >> one) ^ (_MATRIX_A if int(y) & 1 else np.uint64(0))
        self.index = 0

    def raw(self, count: int) -> np.ndarray:
        out = np.empty(count, dtype=np.uint64)
        filled = 0
        while filled < count:
            if self.index >= _N:
                self._twist()
            take = min(count - filled, _N - self.index)
            y = self.mt[self.index:self.index + take].copy()
            y ^= (y >> np.uint64(29)) & np.uint64(0x5555555555555555)
            y ^= (y << np.uint64(17)) & np.uint64(0x71D67FFFEDA60000)
            y ^= (y << np.uint64(37)) & np.uint64(0xFFF7EEE000000000)
            y ^= y >> np.uint64(43)
            out[filled:filled + take] = y
            filled += take
            self.index += take
        return out

    def uniform01(self, count: int) -> np.ndarray:
        """std::uniform_real_distribution<double>(0, 1): one 64-bit word,
        rounded to double, divided by 2^64, kept below 1."""
        x = self.raw(count).astype(np.float64) / 18446744073709551616.0
        x[x >= 1.0] = np.nextafter(1.0, 0.0)
        return x


def splitmix64(x: int) -> int:
    x = (x + 0x9E3779B97F4A7C15) & _MASK
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & _MASK
    return x ^ (x >> 31)


def derive_seed(base_seed: int, stream_tag: int, sequence_index: int = 0) -> int:
    """derive_mcmcmc_seed (mcmcmc_sampler.h:166-172)."""
    mixed = splitmix64((base_seed ^ stream_tag) & _MASK)
    mixed ^= (0x9E3779B97F4A7C15 * (sequence_index + 1)) & _MASK
    return splitmix64(mixed)


def uniform_configurations(seed: int, batch: int, order: int) -> np.ndarray:
    """[batch][order][4] unit vertices, vertex by vertex as
    sample_uniform_vertex_set (mcmcmc_sampler.h:192-198) draws them."""
    return MT19937_64(seed).uniform01(batch * order * 4).reshape(batch, order, 4)


def truncated_geometric_orders(seed: int, batch: int, p: float, n_max: int) -> np.ndarray:
    """Orders 1..n_max with P(n) proportional to p (1-p)^(n-1)."""
    weights = p * (1.0 - p) ** np.arange(n_max)
    cdf = np.cumsum(weights / weights.sum())
    u = MT19937_64(seed).uniform01(batch)
    return (np.searchsorted(cdf, u, side="right") + 1).clip(1, n_max).astype(np.int32)
