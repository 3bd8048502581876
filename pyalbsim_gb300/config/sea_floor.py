"""Seafloor reflectance; fields and defaults as ``alb_sim/config/sea_floor.py:4-16``."""

from dataclasses import dataclass, field


@dataclass(frozen=True)
class SeaFloorConfig:
    albedo: float = field(
        default=0.05, metadata={"description": "Lambertian reflectance of the seafloor"}
    )

    def __post_init__(self):
        if not 0 <= self.albedo <= 1:
            raise ValueError("Albedo must be between 0 and 1")
