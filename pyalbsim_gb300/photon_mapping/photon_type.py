"""Photon-record categories, in the reference's enum order (``alb_sim/photon_mapping/photon_type.py:4-10``).

The integer ``channel`` of each member is the index used by the C ABI and the device
buffers: BOTTOM_REFLECTION=0, SCATTER=1, SURFACE_REFLECTION=2, SURFACE_TRANSMISSION_UP=3.
"""

from enum import Enum, auto


class PhotonType(Enum):
    BOTTOM_REFLECTION = auto()
    SCATTER = auto()
    SURFACE_REFLECTION = auto()
    SURFACE_TRANSMISSION_UP = auto()

    @property
    def channel(self) -> int:
        return self.value - 1


def photon_type_of_channel(channel: int, enum_cls=PhotonType):
    """Map a device channel index to a member of ``enum_cls`` (ours or the reference's)."""
    return list(enum_cls)[channel]
