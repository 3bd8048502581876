"""Dense per-type photon records, as ``alb_sim/photon_mapping/photon_map_data.py:6-15``."""

from dataclasses import dataclass

import numpy as np


@dataclass
class PhotonMapData:
    positions: np.ndarray  # (N, 3) float32
    directions: np.ndarray  # (N, 3) float32
    energies: np.ndarray  # (N,) float32
    times: np.ndarray  # (N,) float32, integrator step of the event
    first_water_interaction: np.ndarray  # (N, 3) float32, NaN when unknown
    seafloor_interaction: np.ndarray  # (N, 3) float32, NaN when unknown
