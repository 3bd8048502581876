"""Options of the GPU engine that have no counterpart in the reference's configs."""

from dataclasses import dataclass
from typing import Optional


@dataclass
class GpuRunOptions:
    """Knobs of the GPU engine.

    rng:        "philox" (counter-based streams keyed by the seed) or "replay"
                (variates supplied by the caller, one stream per photon).
    device:     CUDA device ordinal.
    map_capacity_factor: over-allocation of the photon-map buffers relative to the
                pilot estimate; an overflow is detected and the pass re-run.
    """

    rng: str = "philox"
    device: int = 0
    map_capacity_factor: float = 1.5
    sort_queries: bool = True
    seed: Optional[int] = None
    # precise=True: float64 event geometry and the reference's exact float32 optical-depth
    # rounding (per-photon reproducible against the CPU restatement); precise=False: the
    # float32 tracer, equal in distribution. Replayed variates always use the precise one.
    precise: bool = False
    # adjoint=True (extension): every record and query carries its path score and the
    # gather accumulates d waveform / d (a, b, g, albedo, roughness) beside the waveform
    adjoint: bool = False
