"""Sea-surface settings; fields and defaults as ``alb_sim/config/sea_surface.py:4-19``.

``roughness`` is squared before it enters the GGX distribution
(``alb_sim/physics/reflection/microfacet_brdf.py:125``), so a GGX alpha of a is
``roughness = sqrt(a)``.
"""

from dataclasses import dataclass, field
from typing import Optional


@dataclass(frozen=True)
class SeaSurfaceConfig:
    albedo: float = field(
        default=0.1, metadata={"description": "Diffuse reflectance added to transmission"}
    )
    roughness: float = field(
        default=0.05, metadata={"description": "Microfacet roughness (alpha = roughness^2)"}
    )

    # Extension (the reference's surface is flat): Gaussian surface slopes, std of the slope
    # components; None or 0 keeps the flat surface.
    slope_sigma: Optional[float] = field(
        default=None, metadata={"unit": "rad", "description": "Gaussian surface-slope std; None: flat"}
    )

    def __post_init__(self):
        if not 0 <= self.albedo <= 1:
            raise ValueError("Albedo must be between 0 and 1")
        if self.slope_sigma is not None and not self.slope_sigma >= 0:
            raise ValueError("slope_sigma must be >= 0")
