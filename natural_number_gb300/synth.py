"""Seeded synthetic operands: uniform u64 limbs from SplitMix64.

SplitMix64 (Steele, Lea & Flood 2014): state_k = seed + k * 0x9E3779B97F4A7C15,
output = mix(state_k).  Limb i of an operand drawn with (seed, n) is output i+1
of the stream, so any prefix or slice can be generated independently.  The top
limb is forced nonzero (re-drawn from the stream's next output, or 1), matching
the "top limb nonzero" rule of every benchmark configuration.
"""
from __future__ import annotations

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def splitmix64(seed: int, count: int, start: int = 0) -> np.ndarray:
    """Outputs start+1 .. start+count of the SplitMix64 stream for `seed`."""
    with np.errstate(over="ignore"):
        k = np.arange(start + 1, start + count + 1, dtype=np.uint64)
        return _mix(np.uint64(seed & (2**64 - 1)) + k * _GAMMA)


def limbs(seed: int, n: int) -> np.ndarray:
    """n uniform u64 limbs with a nonzero top limb."""
    if n <= 0:
        raise ValueError("operand needs at least one limb")
    x = splitmix64(seed, n)
    if x[-1] == 0:
        r = splitmix64(seed, 1, start=n)[0]
        x[-1] = r if r != 0 else np.uint64(1)
    return x


def log_uniform_sizes(seed: int, count: int, lo_exp: float, hi_exp: float) -> np.ndarray:
    """floor(2^(lo + (hi-lo)*u)) with u uniform in [0,1) from SplitMix64's top 53 bits."""
    u = (splitmix64(seed, count) >> np.uint64(11)).astype(np.float64) * (1.0 / 2**53)
    return np.floor(np.exp2(lo_exp + (hi_exp - lo_exp) * u)).astype(np.int64)
