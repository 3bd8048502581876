"""GPU engine: one device context per simulation, driving the C ABI pass by pass.

This is the layer the drop-in drivers (``execution.linear``, ``execution.parallel``) and
the ``Simulation`` facade sit on. It owns a ``NativeContext`` (libalbgpu.so) and keeps the
photon counters that turn per-call photon indices into distinct Philox streams.
"""

from __future__ import annotations

import secrets
from typing import Dict, Optional

import numpy as np

from pyalbsim_gb300._native import (
    ALB_OPT_ADJOINT,
    ALB_OPT_KEEP_EXIT_STATES,
    ALB_OPT_KEEP_RECORD_IDS,
    ALB_OPT_PRECISE,
    ALB_OPT_SORT_QUERIES,
    NativeContext,
)
from pyalbsim_gb300.config.gpu import GpuRunOptions
from pyalbsim_gb300.photon_mapping.photon_map_data import PhotonMapData
from pyalbsim_gb300.photon_mapping.photon_type import PhotonType
from pyalbsim_gb300.scene import build_scene
from pyalbsim_gb300.utils.heatmap_result import SampledHeatmapsResult

CHANNELS = list(PhotonType)


def seed_from_rng(rng: Optional[np.random.Generator]) -> int:
    """64-bit Philox key: from the caller's Generator, or random like the reference
    (alb_sim/execution/linear.py:99-100 seeds from secrets when rng is None)."""
    if rng is None:
        return secrets.randbits(64)
    return int(rng.integers(0, 2**63, dtype=np.int64))


class GpuEngine:
    def __init__(self, simulation_config, options: Optional[GpuRunOptions] = None):
        self.options = options or GpuRunOptions()
        self.config = simulation_config
        self.scene = build_scene(simulation_config)
        self.ctx = NativeContext(self.scene, device=self.options.device)
        try:
            self.ctx.set_option(ALB_OPT_SORT_QUERIES, 1 if self.options.sort_queries else 0)
            self.ctx.set_option(ALB_OPT_PRECISE, 1 if self.options.precise else 0)
            if self.options.adjoint:
                self.ctx.set_option(ALB_OPT_ADJOINT, 1)
        except Exception:
            self.ctx.close()  # e.g. the adjoint refused on depth-profiled layers
            raise
        self.n_forward = 0
        self.n_backward = 0
        self._maps_stale = True

    # -- passes ------------------------------------------------------------------------
    def forward(self, n: int, seed: int, first: Optional[int] = None, replay=None):
        """Trace n forward photons and append their records to the photon maps."""
        start = self.n_forward if first is None else first
        self.ctx.trace(True, int(n), seed=seed, first=start, replay=replay)
        self.n_forward += int(n)
        self._maps_stale = True

    def build_maps(self):
        self.ctx.build_maps()
        self._maps_stale = False

    def backward(self, n: int, seed: int, first: Optional[int] = None, replay=None):
        """Trace n backward photons, gather at every event and accumulate the waveform."""
        if self._maps_stale:
            self.build_maps()
        start = self.n_backward if first is None else first
        self.ctx.trace(False, int(n), seed=seed, first=start, replay=replay)
        self.n_backward += int(n)

    # -- results -----------------------------------------------------------------------
    def waveform(self, enum_cls=PhotonType, f64: bool = False) -> Dict:
        return {member: self.ctx.waveform(i, f64=f64) for i, member in enumerate(enum_cls)}

    def waveform_array(self, f64: bool = True) -> np.ndarray:
        return np.stack([self.ctx.waveform(i, f64=f64) for i in range(4)])

    def photon_maps_data(self, enum_cls=PhotonType, data_cls=PhotonMapData) -> Dict:
        out = {}
        for i, member in enumerate(enum_cls):
            if self.ctx.map_size(i) == 0:
                continue
            pos, d, e, t, fwi, sfi, _ = self.ctx.export_map(i)
            out[member] = data_cls(
                positions=pos, directions=d, energies=e, times=t,
                first_water_interaction=fwi, seafloor_interaction=sfi,
            )
        return out

    def heatmaps(self, result_cls=SampledHeatmapsResult) -> Optional[SampledHeatmapsResult]:
        if not self.scene.heatmap_enabled:
            return None
        b = self.scene.heatmap_bins
        w, f, r = self.ctx.heatmaps()
        return result_cls(
            water_heatmap=w.reshape(b, b).astype(np.float32),
            seafloor_heatmap=f.reshape(b, b).astype(np.float32),
            scatter_radius_heatmap=r.reshape(b, b),
        )

    def jacobian(self) -> np.ndarray:
        """d waveform / d (a, b, g, albedo, roughness), float64 [5, channels, nbins]
        (needs GpuRunOptions(adjoint=True))."""
        return self.ctx.jacobian()

    def keep_exit_states(self, on: bool = True):
        self.ctx.set_option(ALB_OPT_KEEP_EXIT_STATES, int(on))

    def keep_record_ids(self, on: bool = True):
        self.ctx.set_option(ALB_OPT_KEEP_RECORD_IDS, int(on))

    def close(self):
        self.ctx.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False
