"""Scene geometry; fields and defaults as ``alb_sim/config/scene.py:4-16``."""

from dataclasses import dataclass, field


@dataclass(frozen=True)
class SceneConfig:
    flying_height: float = field(
        default=135,
        metadata={"unit": "m", "description": "Sensor and laser height above the water"},
    )

    def __post_init__(self):
        if self.flying_height <= 0:
            raise ValueError("Flying height must be positive")
