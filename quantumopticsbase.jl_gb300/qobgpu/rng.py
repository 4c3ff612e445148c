"""Seeded, platform-independent random inputs.

SplitMix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number
generators", OOPSLA 2014) feeds Box-Muller (Box & Muller 1958) to make complex
Gaussian amplitudes.  Written with numpy uint64 arithmetic so the same seed
gives the same arrays on x86 and Arm hosts, for the oracle and the GPU alike.
"""
from __future__ import annotations

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, start: int, n: int) -> np.ndarray:
    """Outputs start+1 .. start+n of the SplitMix64 sequence seeded by ``seed``."""
    with np.errstate(over="ignore"):
        i = np.arange(start + 1, start + n + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


class Rng:
    """A counter-based stream: every draw advances the counter."""

    def __init__(self, seed: int):
        self.seed = int(seed)
        self.counter = 0

    def _raw(self, n: int) -> np.ndarray:
        z = splitmix64(self.seed, self.counter, n)
        self.counter += n
        return z

    def uniform(self, n: int = 1, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        u = (self._raw(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u

    def integers(self, n: int, lo: int, hi: int) -> np.ndarray:
        """Uniform integers in [lo, hi] inclusive."""
        u = self.uniform(n)
        return np.minimum(lo + np.floor(u * (hi - lo + 1)).astype(np.int64), hi)

    def complex_normal(self, n: int) -> np.ndarray:
        u1 = 1.0 - self.uniform(n)  # (0, 1]
        u2 = self.uniform(n)
        r = np.sqrt(-2.0 * np.log(u1))
        return r * np.cos(2 * np.pi * u2) + 1j * r * np.sin(2 * np.pi * u2)

    def ket_data(self, dim: int, dtype=np.complex128) -> np.ndarray:
        """A normalised complex-Gaussian state vector (normalised in FP64)."""
        v = self.complex_normal(dim)
        v /= np.sqrt(np.sum(np.abs(v) ** 2))
        return v.astype(dtype)

    def kets_data(self, dim: int, n: int, dtype=np.complex128) -> np.ndarray:
        """``n`` normalised kets as the columns of a Fortran-ordered dim x n array."""
        out = np.empty((dim, n), dtype=dtype, order="F")
        for c in range(n):
            out[:, c] = self.ket_data(dim, dtype)
        return out
