"""Multi-GPU runs of the multiply path: independent replicas.

A product of two naturals does not shard without an exchange step (every
output limb depends on every input limb through the transform), and the
reference has no multi-device path, so N GPUs run N independent replicas:
rank r multiplies its own operands (seeds offset by r), nothing crosses
between ranks on the data path, and the only collectives are the barrier
around the timed region and one max-reduction of the elapsed time.  The
reported value is the units all ranks processed divided by the slowest
rank's time (weak scaling: per-rank work is fixed as N grows).
"""
from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass(frozen=True)
class Rank:
    rank: int = 0
    world: int = 1
    local: int = 0

    @classmethod
    def from_env(cls) -> "Rank":
        return cls(int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
                   int(os.environ.get("LOCAL_RANK", "0")))

    def seeds(self, seed_a: int, seed_b: int) -> tuple[int, int]:
        """Operand seeds of this rank's replica."""
        return seed_a + self.rank, seed_b + self.rank


def barrier(dist) -> None:
    if dist is not None and dist.is_initialized():
        dist.barrier()


def max_over_ranks(value: float, dist, device: str = "cpu") -> float:
    """The largest `value` over all ranks (identity without a process group);
    `device` is "cuda" under NCCL and "cpu" under gloo."""
    if dist is None or not dist.is_initialized():
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, world: int, slowest_ms: float) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time per step."""
    return world * units_per_rank / (slowest_ms / 1e3)
