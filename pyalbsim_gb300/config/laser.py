"""Laser source settings; fields and defaults as ``alb_sim/config/laser.py:4-47``.

``nadir_angle`` and ``azimuth_angle`` are read in DEGREES by the model
(``alb_sim/physics/models/laser.py:22-33``) although the reference's metadata says rad;
the drop-in keeps that behaviour.
"""

from dataclasses import dataclass, field


@dataclass(frozen=True)
class LaserConfig:
    divergence_angle: float = field(
        default=1e-3, metadata={"unit": "rad", "description": "Beam divergence half-angle"}
    )
    wavelength: float = field(
        default=0.532, metadata={"unit": "µm", "description": "Vacuum wavelength"}
    )
    nadir_angle: float = field(
        default=15.0,
        metadata={"unit": "deg", "description": "Angle of the beam from the -y axis"},
    )
    azimuth_angle: float = field(
        default=0.0,
        metadata={"unit": "deg", "description": "Beam azimuth about y (0 = +x)"},
    )
    pulse_fwhm: float = field(
        default=8.3e-9, metadata={"unit": "s", "description": "Pulse FWHM"}
    )

    def __post_init__(self):
        if self.nadir_angle >= 90:
            raise ValueError("Nadir angle must be below 90 degrees")
