from pyalbsim_gb300.photon_mapping.photon_map_data import PhotonMapData
from pyalbsim_gb300.photon_mapping.photon_type import PhotonType

__all__ = ["PhotonMapData", "PhotonType"]
