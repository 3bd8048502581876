"""Heatmap bundle returned by ``run_parallel`` (``alb_sim/utils/heatmap_result.py:6-14``)."""

from dataclasses import dataclass

import numpy as np


@dataclass
class SampledHeatmapsResult:
    water_heatmap: np.ndarray  # (bins, bins) energy at first-water-interaction points
    seafloor_heatmap: np.ndarray  # (bins, bins) energy at seafloor-interaction points
    scatter_radius_heatmap: np.ndarray  # (bins, bins) surface radius vs seafloor radius counts
