"""Depth profiles for water-layer optical properties.

Drop-in equivalents of the profile objects in ``alb_sim/utils/parameter_profile.py``
(``LinearParameter`` :46-72, ``ExponentialParameter`` :75-99 and
``normalize_number_or_scalar`` :21-43). A layer property is either a plain float or an
object with ``at(t)`` evaluated at the fractional depth ``t`` in [0, 1] of the layer.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Protocol, Union

import numpy as np


class ScalarParameter(Protocol):
    def at(self, t): ...


NumberOrScalar = Union[float, ScalarParameter]


def normalize_number_or_scalar(value):
    """Turn integers into floats, reject booleans, pass profile objects through."""
    if isinstance(value, bool):
        raise TypeError("Boolean is not a valid numeric parameter")
    if isinstance(value, int):
        return float(value)
    return value


@dataclass(frozen=True)
class LinearParameter:
    """Value varying linearly from ``start`` (top of layer) to ``end`` (bottom)."""

    start: float
    end: float

    def at(self, t):
        is_scalar = np.isscalar(t)
        tt = np.asarray(t, dtype=np.float32)
        out = self.start + tt * (self.end - self.start)
        return out.item() if is_scalar else out


@dataclass(frozen=True)
class ExponentialParameter:
    """Value varying log-linearly from ``start`` to ``end`` (both must be positive)."""

    start: float
    end: float

    def __post_init__(self):
        if self.start <= 0 or self.end <= 0:
            raise ValueError("ExponentialProfile requires positive values")

    def at(self, t):
        lo = np.log(self.start)
        hi = np.log(self.end)
        return np.exp(lo + t * (hi - lo))
