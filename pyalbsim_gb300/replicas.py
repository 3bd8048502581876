"""Replicas on several GPUs of one node (the path has no data-path exchange).

Every rank traces its own Philox streams on its own GPU; the only collective is the max of
the ranks' timed durations, taken once after the timed region. The backend is whatever
process group the caller initialised (NCCL on GPUs, gloo in the CPU tests).
"""

from __future__ import annotations

import os
from typing import Tuple


def rank_info() -> Tuple[int, int, int]:
    """(world size, rank, local rank) from the torchrun environment (1, 0, 0 without it)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seed(base: int, rank: int, step: int = 0) -> int:
    """Philox key of a rank's step: base, rank and step in separate bit fields of the 64-bit
    key (base above bit 32, rank in bits 20..31, step below bit 20), so two different
    (base, rank, step) triples never share a stream."""
    if not (0 <= rank < (1 << 12) and 0 <= step < (1 << 20) and 0 <= base < (1 << 32)):
        raise ValueError("replica_seed: base < 2^32, rank < 2^12 and step < 2^20 are required")
    return (base << 32) | (rank << 20) | step


def max_over_ranks(value: float, device: str = "cpu") -> float:
    """Max of a per-rank float over the initialised process group (the value itself when
    torch.distributed is not initialised)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, world: int, ms: float) -> float:
    """Whole-job throughput: every rank processed units_per_rank in at most ms."""
    return world * units_per_rank / (ms / 1e3)
