"""Sea-surface settings; fields and defaults as ``alb_sim/config/sea_surface.py:4-19``.

``roughness`` is squared before it enters the GGX distribution
(``alb_sim/physics/reflection/microfacet_brdf.py:125``), so a GGX alpha of a is
``roughness = sqrt(a)``.
"""

from dataclasses import dataclass, field


@dataclass(frozen=True)
class SeaSurfaceConfig:
    albedo: float = field(
        default=0.1, metadata={"description": "Diffuse reflectance added to transmission"}
    )
    roughness: float = field(
        default=0.05, metadata={"description": "Microfacet roughness (alpha = roughness^2)"}
    )

    def __post_init__(self):
        if not 0 <= self.albedo <= 1:
            raise ValueError("Albedo must be between 0 and 1")
