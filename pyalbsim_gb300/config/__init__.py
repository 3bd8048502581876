"""Configuration dataclasses accepted by the GPU drop-in.

The classes mirror ``alb_sim.config`` field for field (same names, defaults, units and
validation) so that scripts written against the reference keep working after an import
change. The drop-in also accepts the reference's own config objects unchanged: every
consumer reads attributes only.
"""

from pyalbsim_gb300.config.heatmap import HeatmapConfig
from pyalbsim_gb300.config.laser import LaserConfig
from pyalbsim_gb300.config.run import RunConfig
from pyalbsim_gb300.config.scene import SceneConfig
from pyalbsim_gb300.config.sea_floor import SeaFloorConfig
from pyalbsim_gb300.config.sea_surface import SeaSurfaceConfig
from pyalbsim_gb300.config.sensor import SensorConfig
from pyalbsim_gb300.config.simulation import SimulationConfig
from pyalbsim_gb300.config.water import (
    FournierForandConfig,
    TurbidityLayerConfig,
    WaterConfig,
)
from pyalbsim_gb300.config.gpu import GpuRunOptions

__all__ = [
    "FournierForandConfig",
    "GpuRunOptions",
    "HeatmapConfig",
    "LaserConfig",
    "RunConfig",
    "SceneConfig",
    "SeaFloorConfig",
    "SeaSurfaceConfig",
    "SensorConfig",
    "SimulationConfig",
    "TurbidityLayerConfig",
    "WaterConfig",
]
