"""GPU facade of the reference's ``Simulation`` object (alb_sim/core/simulation.py:26-107).

Workers and notebooks of the reference drive ``Simulation(config, rng)`` directly:
``simulate_batch(n, forward=True/False)`` and the attributes ``photon_storage``,
``photon_maps`` and ``return_waveform``. The facade keeps that surface; the attributes
are materialised from the device on access.
"""

from __future__ import annotations

from collections import defaultdict

import numpy as np

from pyalbsim_gb300.engine import GpuEngine, seed_from_rng
from pyalbsim_gb300.photon_mapping.photon_type import PhotonType


class _MapIndexView:
    """Stand-in for PhotonMapIndex: ``.data`` is the PhotonMapData of one type."""

    def __init__(self, data):
        self.data = data


class _StorageView:
    """Stand-in for PhotonStorage: one concatenated array per type in each dict."""

    def __init__(self, maps):
        self.positions = defaultdict(list)
        self.directions = defaultdict(list)
        self.energies = defaultdict(list)
        self.times = defaultdict(list)
        self.first_water_interaction = defaultdict(list)
        self.seafloor_interaction = defaultdict(list)
        for t, m in maps.items():
            self.positions[t].append(m.positions)
            self.directions[t].append(m.directions)
            self.energies[t].append(m.energies)
            self.times[t].append(m.times)
            self.first_water_interaction[t].append(m.first_water_interaction)
            self.seafloor_interaction[t].append(m.seafloor_interaction)


class Simulation:
    def __init__(self, config, rng: np.random.Generator):
        self.rng = rng
        self.engine = GpuEngine(config)
        self.model = self.engine.scene
        self._seed = seed_from_rng(rng)
        self.current_step = 0

    def simulate_batch(self, num_photons: int, *, forward: bool):
        if forward:
            self.engine.forward(num_photons, self._seed)
        else:
            self.engine.backward(num_photons, self._seed)
        self.current_step = self.model.total_substeps

    @property
    def return_waveform(self):
        return self.engine.waveform(enum_cls=PhotonType)

    @property
    def photon_maps(self):
        return {t: _MapIndexView(d) for t, d in self.engine.photon_maps_data().items()}

    @property
    def photon_storage(self):
        return _StorageView(self.engine.photon_maps_data())
