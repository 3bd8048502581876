"""Top-level simulation settings; fields and defaults as ``alb_sim/config/simulation.py:12-60``."""

from dataclasses import dataclass, field
from typing import Optional, Tuple

from pyalbsim_gb300.config.heatmap import HeatmapConfig
from pyalbsim_gb300.config.laser import LaserConfig
from pyalbsim_gb300.config.scene import SceneConfig
from pyalbsim_gb300.config.sea_floor import SeaFloorConfig
from pyalbsim_gb300.config.sea_surface import SeaSurfaceConfig
from pyalbsim_gb300.config.sensor import SensorConfig
from pyalbsim_gb300.config.water import WaterConfig


@dataclass(frozen=True)
class SimulationConfig:
    sample_multiplier: int = field(
        default=10, metadata={"description": "Integrator sub-steps per waveform sample"}
    )
    photon_mapping_k: int = field(
        default=100, metadata={"description": "Neighbours per photon-map density estimate"}
    )
    scene: SceneConfig = field(default_factory=SceneConfig)
    water: WaterConfig = field(default_factory=WaterConfig)
    laser: LaserConfig = field(default_factory=LaserConfig)
    sensor: SensorConfig = field(default_factory=SensorConfig)
    sea_floor: SeaFloorConfig = field(default_factory=SeaFloorConfig)
    sea_surface: SeaSurfaceConfig = field(default_factory=SeaSurfaceConfig)
    heatmap: HeatmapConfig = field(default_factory=HeatmapConfig)
    # Extension (no counterpart in the reference): density estimates over every photon-map
    # record within this radius (m) instead of the k nearest; None keeps the k-NN gather.
    gather_radius: Optional[float] = field(
        default=None, metadata={"unit": "m", "description": "Fixed gather radius; None: k nearest"}
    )

    # Extension: gated waveform window (start, length) in seconds after emission; the
    # waveforms then hold only the bins of that window. None keeps the whole timeline.
    waveform_gate: Optional[Tuple[float, float]] = field(
        default=None, metadata={"unit": "s", "description": "Waveform window (start, length); None: all"}
    )

    def __post_init__(self):
        if self.gather_radius is not None and not self.gather_radius > 0:
            raise ValueError("gather_radius must be positive (None selects the k-NN gather)")
        if self.waveform_gate is not None:
            start, length = (float(x) for x in self.waveform_gate)
            if start < 0 or not length > 0:
                raise ValueError("waveform_gate needs start >= 0 and length > 0")
