"""Sampled-heatmap settings; fields and defaults as ``alb_sim/config/heatmap.py:4-33``."""

from dataclasses import dataclass, field


@dataclass(frozen=True)
class HeatmapConfig:
    enabled: bool = field(
        default=True,
        metadata={"description": "Accumulate sampled-energy heatmaps in the backward pass"},
    )
    bins: int = field(
        default=200, metadata={"description": "Bins per axis of every heatmap"}
    )
    water_extent: float = field(
        default=1.0,
        metadata={"unit": "m", "description": "Half-width of the water-surface heatmap"},
    )
    seafloor_extent: float = field(
        default=10.0,
        metadata={"unit": "m", "description": "Half-width of the seafloor heatmap"},
    )
