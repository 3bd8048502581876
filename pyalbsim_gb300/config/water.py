"""Water-column settings; fields, defaults and validation as ``alb_sim/config/water.py:9-125``.

A ``TurbidityLayerConfig`` property may be a float or a depth profile
(``pyalbsim_gb300.utils.parameter_profile``). When neither ``num_sublayers`` nor
``sublayer_dz`` is given the layer is rejected; otherwise ``num_sublayers`` defaults to
``max(2, ceil(height / sublayer_dz))`` as in the reference (``water.py:118-125``).
"""

from dataclasses import dataclass, field
from typing import Optional, Tuple

import numpy as np

from pyalbsim_gb300.utils.parameter_profile import (
    NumberOrScalar,
    normalize_number_or_scalar,
)


@dataclass(frozen=True)
class FournierForandConfig:
    refractive_index_ratio: float = field(
        default=1.1, metadata={"description": "Particle / water refractive index (real)"}
    )
    junge_slope: float = field(
        default=3.62, metadata={"description": "Junge slope of the particle size spectrum"}
    )


@dataclass(frozen=True)
class TurbidityLayerConfig:
    height: float = field(default=3, metadata={"unit": "m", "description": "Thickness"})
    scattering_coefficient: NumberOrScalar = field(
        default=2.5, metadata={"unit": "1/m", "description": "Scattering coefficient b"}
    )
    absorption_coefficient: NumberOrScalar = field(
        default=0.169, metadata={"unit": "1/m", "description": "Absorption coefficient a"}
    )
    salinity: NumberOrScalar = field(
        default=37, metadata={"unit": "ppt", "description": "Salinity"}
    )
    refractive_index: NumberOrScalar = field(
        default=1.33334, metadata={"description": "Refractive index of the water"}
    )
    fournier_forand_parameters: FournierForandConfig = field(
        default_factory=FournierForandConfig
    )
    sublayer_dz: Optional[float] = field(
        default=0.05, metadata={"unit": "m", "description": "Sub-layer thickness"}
    )
    num_sublayers: Optional[int] = field(
        default=None, metadata={"description": "Number of sub-layers of the depth LUT"}
    )
    # Extension (no counterpart in the reference): Henyey-Greenstein scattering with this
    # asymmetry parameter in place of the Fournier-Forand phase function (None: FF).
    henyey_greenstein_g: Optional[float] = field(
        default=None, metadata={"description": "HG asymmetry g in (-1, 1); None selects Fournier-Forand"}
    )

    def __post_init__(self):
        g = self.henyey_greenstein_g
        if g is not None and (not -1.0 < float(g) < 1.0 or g == 0.0):
            raise ValueError("henyey_greenstein_g must lie in (-1, 1) and be non-zero")
        if self.height <= 0:
            raise ValueError("Layer height must be positive")
        for name in (
            "scattering_coefficient",
            "absorption_coefficient",
            "salinity",
            "refractive_index",
        ):
            object.__setattr__(
                self, name, normalize_number_or_scalar(getattr(self, name))
            )
        if self.num_sublayers is None:
            if self.sublayer_dz is None:
                raise ValueError("Either sublayer_dz or num_sublayers must be provided")
            object.__setattr__(
                self,
                "num_sublayers",
                max(2, int(np.ceil(self.height / self.sublayer_dz))),
            )


@dataclass(frozen=True)
class WaterConfig:
    layers: Tuple[TurbidityLayerConfig, ...] = field(
        default_factory=lambda: (TurbidityLayerConfig(),)
    )
