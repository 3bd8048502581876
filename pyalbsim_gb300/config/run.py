"""Batching settings; fields and defaults as ``alb_sim/config/run.py:4-36``.

On the GPU the batches of one pass are traced in one launch sequence, so the totals
``photons_per_batch_* x batches_*`` are what matter; ``processes`` is accepted and ignored.
"""

from dataclasses import dataclass, field


@dataclass
class RunConfig:
    photons_per_batch_forward: int = field(
        default=10_000, metadata={"description": "Photons per forward batch"}
    )
    photons_per_batch_backward: int = field(
        default=5_000, metadata={"description": "Photons per backward batch"}
    )
    batches_forward: int = field(
        default=10, metadata={"description": "Number of forward batches"}
    )
    batches_backward: int = field(
        default=5, metadata={"description": "Number of backward batches"}
    )
    processes: int = field(
        default=8,
        metadata={"description": "Worker processes of the CPU reference (unused on GPU)"},
    )
