"""Receiver settings; fields and defaults as ``alb_sim/config/sensor.py:4-33``."""

from dataclasses import dataclass, field


@dataclass(frozen=True)
class SensorConfig:
    aperture_radius: float = field(
        default=0.1, metadata={"unit": "m", "description": "Telescope aperture radius"}
    )
    field_of_view: float = field(
        default=5e-3, metadata={"unit": "rad", "description": "Field-of-view half-angle"}
    )
    sample_rate: int = field(
        default=int(2e9), metadata={"unit": "Hz", "description": "Waveform sample rate"}
    )

    def __post_init__(self):
        if self.aperture_radius < 0:
            raise ValueError("Aperture radius must be positive")
