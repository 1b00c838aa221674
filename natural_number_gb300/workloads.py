"""Synthetic workloads on the device.

uneven_products(): the batched uneven-size multiply workload — `count`
independent products whose operand lengths are drawn independently,
log-uniformly in [2^lo, 2^hi] limbs, with uniform u64 limbs (SplitMix64,
top limb nonzero).  Operands and outputs live in a few large device buffers;
two nn_mul_job arrays point into them (one output region for the batched
path, one for the one-product-per-launch path) so results can be compared.
"""
from __future__ import annotations

import numpy as np

from . import MulJob
from .synth import limbs, log_uniform_sizes


class UnevenProducts:
    def __init__(self, count: int = 4096, lo: float = 6, hi: float = 18, seed: int = 3, device: str = "cuda"):
        import torch
        self.count = count
        self.sa = log_uniform_sizes(seed, count, lo, hi).astype(np.uint64)
        self.sb = log_uniform_sizes(seed + 1, count, lo, hi).astype(np.uint64)
        self.sa = np.maximum(self.sa, 1)
        self.sb = np.maximum(self.sb, 1)
        oa = np.concatenate([[0], np.cumsum(self.sa)]).astype(np.int64)
        ob = np.concatenate([[0], np.cumsum(self.sb)]).astype(np.int64)
        oo = np.concatenate([[0], np.cumsum(self.sa + self.sb)]).astype(np.int64)
        self.limbs_total = int(oo[-1])
        ha = np.empty(int(oa[-1]), dtype=np.uint64)
        hb = np.empty(int(ob[-1]), dtype=np.uint64)
        for j in range(count):
            ha[oa[j]:oa[j + 1]] = limbs(seed * 1000003 + 2 * j, int(self.sa[j]))
            hb[ob[j]:ob[j + 1]] = limbs(seed * 1000003 + 2 * j + 1, int(self.sb[j]))
        self.host_a, self.host_b = ha, hb
        self.a = torch.from_numpy(ha).to(device)
        self.b = torch.from_numpy(hb).to(device)
        self.out_batch = torch.zeros(self.limbs_total, dtype=torch.uint64, device=device)
        self.out_plain = torch.zeros(self.limbs_total, dtype=torch.uint64, device=device)
        self.offsets = (oa, ob, oo)
        pa, pb = self.a.data_ptr(), self.b.data_ptr()
        self.jobs_batch = (MulJob * count)()
        self.jobs_plain = (MulJob * count)()
        for j in range(count):
            args = (pa + 8 * int(oa[j]), int(self.sa[j]), pb + 8 * int(ob[j]), int(self.sb[j]))
            self.jobs_batch[j] = MulJob(args[0], args[1], args[2], args[3], self.out_batch.data_ptr() + 8 * int(oo[j]))
            self.jobs_plain[j] = MulJob(args[0], args[1], args[2], args[3], self.out_plain.data_ptr() + 8 * int(oo[j]))

    def operands(self, j: int) -> tuple[np.ndarray, np.ndarray]:
        oa, ob, _ = self.offsets
        return self.host_a[oa[j]:oa[j + 1]], self.host_b[ob[j]:ob[j + 1]]

    def product(self, j: int, which: str = "batch") -> np.ndarray:
        _, _, oo = self.offsets
        t = self.out_batch if which == "batch" else self.out_plain
        return t[int(oo[j]):int(oo[j + 1])].cpu().numpy()

    def ntt_fraction(self, threshold: int = 384, balanced: int = 0) -> float:
        """Share of products a batch sends down the NTT route: the shorter
        operand at least `threshold` limbs, and at least `balanced` when the
        longer is at most twice the shorter."""
        mn, mx = np.minimum(self.sa, self.sb), np.maximum(self.sa, self.sb)
        school = (mn < threshold) | ((mn < balanced) & (mx <= 2 * mn))
        return float(np.mean(~school))
