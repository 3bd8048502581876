"""Named workloads: the large single-instance scene and the small reference-runnable one.

large: 400 m altitude, 20 m water, a = 0.10, b = 0.40 (FF phase unless hg is given), GGX
alpha 0.10, albedo 0.20, FOV 50 mrad, 0.05 ns bins (2e10 Hz).
small: 400 m altitude, 5 m water, a = 0.05, b = 0.20, GGX alpha 0.05, albedo 0.15,
FOV 20 mrad, 0.1 ns bins (1e10 Hz).
Both: 532 nm, nadir incidence, 3 ns FWHM pulse, 1 mrad divergence, n_water 1.34, heatmaps off.
"""

from __future__ import annotations

from typing import Optional

import numpy as np


def _config(height, a, b, fov, rate, albedo, ggx_alpha, hg: Optional[float], radius: Optional[float] = None):
    from pyalbsim_gb300.config import (
        HeatmapConfig, LaserConfig, SceneConfig, SeaFloorConfig, SeaSurfaceConfig, SensorConfig,
        SimulationConfig, TurbidityLayerConfig, WaterConfig,
    )

    return SimulationConfig(
        scene=SceneConfig(flying_height=400.0),
        water=WaterConfig(layers=(TurbidityLayerConfig(
            height=height, absorption_coefficient=a, scattering_coefficient=b, refractive_index=1.34,
            henyey_greenstein_g=hg),)),
        laser=LaserConfig(divergence_angle=1e-3, nadir_angle=0.0, pulse_fwhm=3e-9),
        sensor=SensorConfig(field_of_view=fov, sample_rate=int(rate)),
        sea_floor=SeaFloorConfig(albedo=albedo),
        sea_surface=SeaSurfaceConfig(roughness=float(np.sqrt(ggx_alpha))),
        heatmap=HeatmapConfig(enabled=False),
        gather_radius=radius,
    )


def large(hg: Optional[float] = None, radius: Optional[float] = None):
    return _config(20.0, 0.10, 0.40, 50e-3, 2e10, 0.20, 0.10, hg, radius)


def small(hg: Optional[float] = None, radius: Optional[float] = None):
    return _config(5.0, 0.05, 0.20, 20e-3, 1e10, 0.15, 0.05, hg, radius)


def workload_config(name: str, hg: Optional[float] = None):
    if name == "large":
        return large(hg)
    if name == "small":
        return small(hg)
    raise ValueError(name)
