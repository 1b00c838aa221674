"""Shared helpers for the GPU parity tests."""
import hashlib

import numpy as np

P = [27 << 56 | 1, 58 << 56 | 1, 87 << 56 | 1]


def digest(x):
    x = np.ascontiguousarray(x, dtype="<u8")
    return {"n": int(x.size), "sha256": hashlib.sha256(x.tobytes()).hexdigest()}


def to_dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64)).to("cuda")


def empty_dev(n):
    import torch
    return torch.zeros(max(int(n), 1), dtype=torch.uint64, device="cuda")


def to_host(t, n=None):
    import torch
    torch.cuda.synchronize()
    a = t.cpu().numpy()
    return a if n is None else a[:n]


def normalize(x):
    n = len(x)
    while n > 1 and x[n - 1] == 0:
        n -= 1
    return x[:n]


def mod_checks(limbs):
    """(value mod 2^64-1, value mod 2^64+1) of a little-endian limb array,
    computed with numpy in a size-independent way (B = 2^64 is 1 and -1)."""
    x = np.ascontiguousarray(limbs, dtype=np.uint64)
    lo = (x & np.uint64(0xFFFFFFFF)).astype(np.uint64)
    hi = (x >> np.uint64(32)).astype(np.uint64)

    def wsum(v):  # exact sum of < 2^32 values as Python int
        return int(v.astype(np.uint64).sum(dtype=np.uint64)) if v.size < (1 << 31) else int(
            sum(int(c.sum(dtype=np.uint64)) for c in np.array_split(v, 64)))

    s_all = wsum(lo) + (wsum(hi) << 32)
    even_lo, odd_lo = lo[0::2], lo[1::2]
    even_hi, odd_hi = hi[0::2], hi[1::2]
    s_even = wsum(even_lo) + (wsum(even_hi) << 32)
    s_odd = wsum(odd_lo) + (wsum(odd_hi) << 32)
    m1 = (1 << 64) - 1
    m2 = (1 << 64) + 1
    return s_all % m1, (s_even - s_odd) % m2
