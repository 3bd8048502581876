"""Generate the golden fixtures under tests/golden/ by running the reference simulator.

Run where the reference is importable: ``ALB_REFERENCE_SRC`` names the directory that holds
its ``alb_sim`` package, else the copy installed into ``baseline/_ref`` (``python -m pip
install --no-deps --target baseline/_ref <reference checkout>``) is used. The GPU tests never run this script: the fixtures it writes
are committed. Nothing here restates the reference's physics; the script only drives the
reference's own objects and records what they do:

* a proxy ``numpy.random.Generator`` logs every draw and attributes it to photon ids
  (the ids travel with a ``PhotonWrapper`` subclass through ``subset``/``copy``);
* thin overrides of ``Simulation`` methods (calling the originals) set the current id
  context, capture the final photon state and log photon-map record ids;
* a numpy proxy in ``alb_sim.core.simulation`` captures each gather's contributions so
  that a float64 re-accumulation of the waveform can be stored beside the reference's
  own float32 one.

Fixtures:
  kat_physics.npz      known-answer values of the reference's physics functions
  fd_ref.npz           reference waveforms at seafloor albedo and surface roughness +- h
                       (common-random-number differences of the reference itself)
  replay_<name>.npz    per-photon variate streams, photon maps, exit states, queries and
                       waveforms of a small reference run
  knn.npz              scipy KDTree k-nearest-neighbour answers on clustered maps
  stats_small.npz      per-bin mean / standard error over independent reference runs
  stats_cfg0.npz       the same for 32 run_linear calls at the config-0 geometry

Usage: python tests/golden/make_golden.py [kat|replay|knn|stats|stats_cfg0|fd_ref|all]
"""

from __future__ import annotations

import multiprocessing
import os
import sys
import time
from types import SimpleNamespace

import numpy as np

OUT_DIR = os.path.dirname(os.path.abspath(__file__))
REF_SRC = os.environ.get("ALB_REFERENCE_SRC") or os.path.join(
    os.path.dirname(os.path.dirname(OUT_DIR)), "baseline", "_ref")
if not os.path.isdir(os.path.join(REF_SRC, "alb_sim")):
    sys.exit(f"make_golden: no alb_sim package under {REF_SRC}; set ALB_REFERENCE_SRC")

sys.path.insert(0, REF_SRC)
sys.modules.setdefault("multiprocess", multiprocessing)

import alb_sim.core.simulation as core_sim  # noqa: E402
from alb_sim.config.heatmap import HeatmapConfig  # noqa: E402
from alb_sim.config.laser import LaserConfig  # noqa: E402
from alb_sim.config.scene import SceneConfig  # noqa: E402
from alb_sim.config.sea_floor import SeaFloorConfig  # noqa: E402
from alb_sim.config.sea_surface import SeaSurfaceConfig  # noqa: E402
from alb_sim.config.sensor import SensorConfig  # noqa: E402
from alb_sim.config.simulation import SimulationConfig  # noqa: E402
from alb_sim.config.water import TurbidityLayerConfig, WaterConfig  # noqa: E402
from alb_sim.photon_mapping.build_photon_map_data import build_photon_map_data  # noqa: E402
from alb_sim.photon_mapping.photon_map_index import PhotonMapIndex  # noqa: E402
from alb_sim.photon_mapping.photon_type import PhotonType  # noqa: E402
from alb_sim.utils.photon_wrapper import PhotonWrapper  # noqa: E402
from alb_sim.utils.parameter_profile import ExponentialParameter, LinearParameter  # noqa: E402

TYPES = list(PhotonType)  # channel order: BOTTOM, SCATTER, SURFACE_REFLECTION, TRANSMISSION_UP


# ----------------------------------------------------------------------------------
# id-carrying wrapper and recording RNG
# ----------------------------------------------------------------------------------


class IdWrapper(PhotonWrapper):
    ids: np.ndarray = None

    def _with_ids(self, other, ids):
        out = IdWrapper(**{f: getattr(other, f) for f in PhotonWrapper.__dataclass_fields__})
        out.ids = ids
        return out

    def subset(self, idx):
        return self._with_ids(PhotonWrapper.subset(self, idx), self._ids()[idx])

    def copy(self):
        return self._with_ids(PhotonWrapper.copy(self), self._ids().copy())

    def _ids(self):
        if self.ids is None:
            self.ids = np.arange(len(self.energies))
        return self.ids


class Recorder:
    """Per-photon variate streams of one pass."""

    def __init__(self):
        self.streams = None
        self.ctx = None
        self.queue = []
        self.rayleigh_cut = None
        self.rayleigh_next = 0

    def start_pass(self, n):
        self.streams = [[] for _ in range(n)]
        self.ctx = np.arange(n)
        self.queue = []
        self.rayleigh_next = 0

    def take(self, values):
        values = np.asarray(values)
        ids = self.queue.pop(0) if self.queue else self.ctx
        if values.ndim == 0:
            raise RuntimeError("scalar draw not expected")
        if len(values) != len(ids):
            raise RuntimeError(f"draw of {len(values)} for {len(ids)} photons")
        for j, pid in enumerate(ids):
            row = values[j]
            if np.ndim(row) == 0:
                self.streams[pid].append(float(row))
            else:
                self.streams[pid].extend(float(x) for x in row)

    def take_rayleigh(self, values):
        accepted = values[values <= self.rayleigh_cut]
        for v in accepted:
            if self.rayleigh_next < len(self.ctx):
                self.streams[self.ctx[self.rayleigh_next]].append(float(v))
                self.rayleigh_next += 1


class RecordingRNG:
    def __init__(self, seed, recorder):
        self._g = np.random.default_rng(seed)
        self.rec = recorder

    def random(self, size=None):
        v = self._g.random(size)
        self.rec.take(v)
        return v

    def uniform(self, low=0.0, high=1.0, size=None):
        v = self._g.uniform(low, high, size)
        self.rec.take(v)
        return v

    def normal(self, loc=0.0, scale=1.0, size=None):
        v = self._g.normal(loc, scale, size)
        self.rec.take(v)
        return v

    def rayleigh(self, scale=1.0, size=None):
        v = self._g.rayleigh(scale, size)
        self.rec.take_rayleigh(v)
        return v


# ----------------------------------------------------------------------------------
# numpy proxy capturing the gather's np.add.at calls
# ----------------------------------------------------------------------------------


class GatherLog:
    def __init__(self):
        self.shadow = {}
        self.calls = []


class _AddProxy:
    def __init__(self, log):
        self.log = log

    def __call__(self, *a, **k):
        return np.add(*a, **k)

    def at(self, arr, idx, vals):
        np.add.at(arr, idx, vals)
        key = id(arr)
        if key in self.log.shadow:
            np.add.at(self.log.shadow[key], idx, np.asarray(vals, dtype=np.float64))
            self.log.calls.append((key, float(np.sum(np.asarray(vals, np.float64)))))


class NpProxy:
    def __init__(self, log):
        self._add = _AddProxy(log)

    def __getattr__(self, name):
        if name == "add":
            return self._add
        return getattr(np, name)


# ----------------------------------------------------------------------------------
# recording simulation (overrides call the originals)
# ----------------------------------------------------------------------------------


class RecordingSimulation(core_sim.Simulation):
    def __init__(self, config, rng, recorder, glog):
        super().__init__(config, rng)
        self.rec = recorder
        self.glog = glog
        self.final_wrapper = None
        self.map_ids = {t: [] for t in TYPES}
        self.queries = []
        self.shadow = {}
        for t, arr in self.return_waveform.items():
            self.shadow[t] = np.zeros(len(arr), dtype=np.float64)
            glog.shadow[id(arr)] = self.shadow[t]

    def simulate_batch(self, num_photons, *, forward):
        self.rec.start_pass(num_photons)
        self.rec.rayleigh_cut = self.model.laser.divergence_angle
        self.final_wrapper = None
        return super().simulate_batch(num_photons, forward=forward)

    def simulate_photon_step(self, wrapper, *, forward):
        if self.final_wrapper is None:
            self.final_wrapper = wrapper
        return super().simulate_photon_step(wrapper, forward=forward)

    def handle_water(self, subset, next_positions, *, forward):
        self.rec.ctx = subset._ids()
        return super().handle_water(subset, next_positions, forward=forward)

    def handle_enter(self, subset, next_positions, *, forward):
        self.rec.ctx = subset._ids()
        return super().handle_enter(subset, next_positions, forward=forward)

    def handle_exit(self, subset, next_positions, *, forward):
        self.rec.ctx = subset._ids()
        return super().handle_exit(subset, next_positions, forward=forward)

    def handle_seafloor(self, subset, next_positions, *, forward):
        self.rec.ctx = subset._ids()
        return super().handle_seafloor(subset, next_positions, forward=forward)

    def store_photons(self, wrapper, photon_type):
        self.rec.ctx = wrapper._ids()
        self.map_ids[photon_type].append(wrapper._ids().copy())
        return super().store_photons(wrapper, photon_type)

    def sample_photons(self, wrapper, photon_type):
        self.rec.ctx = wrapper._ids()
        n0 = len(self.glog.calls)
        out = super().sample_photons(wrapper, photon_type)
        sums = [c[1] for c in self.glog.calls[n0:]]
        for j in range(len(wrapper.energies)):
            self.queries.append(
                (
                    TYPES.index(photon_type),
                    int(wrapper._ids()[j]),
                    *np.asarray(wrapper.positions[j], np.float64),
                    *np.asarray(wrapper.directions[j], np.float64),
                    float(wrapper.energies[j]),
                    float(wrapper.time_deltas[j]),
                    sums[j],
                )
            )
        return out


def _install_scatter_queue(sim, recorder):
    """Per-layer scatter draws: queue one id subset per layer draw (two draws per layer)."""
    water = sim.model.water
    orig = water.sample_scattering_directions_by_depth

    def wrapped(depths, incoming, rng):
        idx = water.layer_index(depths)
        ctx = recorder.ctx
        for layer in range(len(water.layers)):
            ids = ctx[idx == layer]
            recorder.queue.extend([ids, ids])
        return orig(depths, incoming, rng)

    water.sample_scattering_directions_by_depth = wrapped


def _streams_to_csr(streams):
    lengths = np.array([len(s) for s in streams], dtype=np.int64)
    offsets = np.zeros(len(streams) + 1, dtype=np.int64)
    np.cumsum(lengths, out=offsets[1:])
    flat = np.array([x for s in streams for x in s], dtype=np.float64)
    return offsets, flat


def _state_arrays(prefix, w):
    return {
        f"{prefix}_pos": np.asarray(w.positions, np.float64),
        f"{prefix}_dir": np.asarray(w.directions, np.float64),
        f"{prefix}_energy": np.asarray(w.energies, np.float32),
        f"{prefix}_tau": np.asarray(w.optical_depth, np.float32),
        f"{prefix}_tau_target": np.asarray(w.optical_depth_target, np.float32),
        f"{prefix}_time": np.asarray(w.time_deltas, np.float32),
        f"{prefix}_fwi": np.asarray(w.first_water_interaction, np.float32),
        f"{prefix}_sfi": np.asarray(w.seafloor_interaction, np.float32),
    }


def _prof(v):
    """(kind, start, end) of a layer property: 0 constant, 1 linear, 2 exponential."""
    if isinstance(v, float):
        return (0.0, v, v)
    if isinstance(v, LinearParameter):
        return (1.0, float(v.start), float(v.end))
    if isinstance(v, ExponentialParameter):
        return (2.0, float(v.start), float(v.end))
    raise TypeError(type(v))


def _start(v):
    return v if isinstance(v, float) else float(v.start)


def config_fields(cfg):
    """Flatten a SimulationConfig into npz scalars (layer properties may be profiles)."""
    out = {
        "cfg_sample_multiplier": cfg.sample_multiplier,
        "cfg_k": cfg.photon_mapping_k,
        "cfg_flying_height": cfg.scene.flying_height,
        "cfg_divergence": cfg.laser.divergence_angle,
        "cfg_wavelength": cfg.laser.wavelength,
        "cfg_nadir": cfg.laser.nadir_angle,
        "cfg_azimuth": cfg.laser.azimuth_angle,
        "cfg_pulse_fwhm": cfg.laser.pulse_fwhm,
        "cfg_aperture": cfg.sensor.aperture_radius,
        "cfg_fov": cfg.sensor.field_of_view,
        "cfg_sample_rate": cfg.sensor.sample_rate,
        "cfg_floor_albedo": cfg.sea_floor.albedo,
        "cfg_surface_albedo": cfg.sea_surface.albedo,
        "cfg_roughness": cfg.sea_surface.roughness,
        "cfg_heatmap_enabled": int(cfg.heatmap.enabled),
        "cfg_heatmap_bins": cfg.heatmap.bins,
        "cfg_heatmap_water_extent": cfg.heatmap.water_extent,
        "cfg_heatmap_seafloor_extent": cfg.heatmap.seafloor_extent,
    }
    layers = cfg.water.layers
    out["cfg_layer_height"] = np.array([l.height for l in layers], np.float64)
    out["cfg_layer_a"] = np.array([_start(l.absorption_coefficient) for l in layers], np.float64)
    out["cfg_layer_b"] = np.array([_start(l.scattering_coefficient) for l in layers], np.float64)
    out["cfg_layer_salinity"] = np.array([_start(l.salinity) for l in layers], np.float64)
    out["cfg_layer_n"] = np.array([_start(l.refractive_index) for l in layers], np.float64)
    # [layer, (a, b, salinity, n), (kind, start, end)] and the LUT size
    out["cfg_layer_prof"] = np.array(
        [[_prof(l.absorption_coefficient), _prof(l.scattering_coefficient), _prof(l.salinity),
          _prof(l.refractive_index)] for l in layers], np.float64)
    out["cfg_layer_nsub"] = np.array([l.num_sublayers for l in layers], np.int64)
    out["cfg_layer_junge"] = np.array(
        [l.fournier_forand_parameters.junge_slope for l in layers], np.float64
    )
    out["cfg_layer_nratio"] = np.array(
        [l.fournier_forand_parameters.refractive_index_ratio for l in layers], np.float64
    )
    return out


def run_recorded(cfg, n_fwd, n_bwd, seed):
    recorder = Recorder()
    glog = GatherLog()
    core_sim.PhotonWrapper = IdWrapper
    core_sim.np = NpProxy(glog)
    try:
        rng = RecordingRNG(seed, recorder)
        sim = RecordingSimulation(cfg, rng, recorder, glog)
        _install_scatter_queue(sim, recorder)
        out = {}
        t0 = time.time()
        sim.simulate_batch(n_fwd, forward=True)
        out["fwd_offsets"], out["fwd_stream"] = _streams_to_csr(recorder.streams)
        out.update(_state_arrays("fwd_final", sim.final_wrapper))
        maps = build_photon_map_data(sim.photon_storage)
        for t in TYPES:
            c = TYPES.index(t)
            if t in maps:
                m = maps[t]
                out[f"map{c}_pos"] = m.positions
                out[f"map{c}_dir"] = m.directions
                out[f"map{c}_energy"] = m.energies
                out[f"map{c}_time"] = m.times
                out[f"map{c}_fwi"] = m.first_water_interaction
                out[f"map{c}_sfi"] = m.seafloor_interaction
                out[f"map{c}_ids"] = np.concatenate(sim.map_ids[t]).astype(np.int64)
                sim.photon_maps[t] = PhotonMapIndex(m)
        t1 = time.time()
        sim.simulate_batch(n_bwd, forward=False)
        t2 = time.time()
        out["bwd_offsets"], out["bwd_stream"] = _streams_to_csr(recorder.streams)
        out.update(_state_arrays("bwd_final", sim.final_wrapper))
        out["queries"] = np.array(sim.queries, dtype=np.float64).reshape(-1, 11)  # kind, id, pos3, dir3, E, t, sum
        out["waveform32"] = np.stack([sim.return_waveform[t] for t in TYPES])
        out["waveform64"] = np.stack([sim.shadow[t] for t in TYPES])
        if cfg.heatmap.enabled:
            out["heat_water"] = sim.sampled_water_heatmap
            out["heat_floor"] = sim.sampled_seafloor_heatmap
            out["heat_radius"] = sim.scatter_radius_heatmap
        out["steps"] = sim.model.steps
        out["n_fwd"] = n_fwd
        out["n_bwd"] = n_bwd
        out["seed"] = seed
        out["ref_seconds_fwd"] = t1 - t0
        out["ref_seconds_bwd"] = t2 - t1
        # tau targets exactly as the reference forms them: -log(float32(U)) in float32
        for p in ("fwd", "bwd"):
            s = out[f"{p}_stream"]
            with np.errstate(divide="ignore"):
                out[f"{p}_stream_tau"] = -np.log(s.astype(np.float32))
        out.update(config_fields(cfg))
        for i, layer in enumerate(sim.model.water.layers):
            if hasattr(layer, "_z_lut"):  # profiled layer: the reference's attenuation LUT
                out[f"lut{i}_z"] = layer._z_lut
                out[f"lut{i}_alpha"] = layer._lidar_alpha_lut
        return out
    finally:
        core_sim.PhotonWrapper = PhotonWrapper
        core_sim.np = np


# ----------------------------------------------------------------------------------
# fixture sets
# ----------------------------------------------------------------------------------


def small_config(k=32, heatmap=True, nadir=10.0, azimuth=30.0):
    return SimulationConfig(
        photon_mapping_k=k,
        scene=SceneConfig(flying_height=10.0),
        water=WaterConfig(
            layers=(
                TurbidityLayerConfig(
                    height=2.0,
                    absorption_coefficient=0.1,
                    scattering_coefficient=1.0,
                    refractive_index=1.34,
                ),
            )
        ),
        laser=LaserConfig(
            divergence_angle=5e-3, nadir_angle=nadir, azimuth_angle=azimuth, pulse_fwhm=3e-9
        ),
        sensor=SensorConfig(aperture_radius=0.1, field_of_view=50e-3, sample_rate=int(1e9)),
        sea_floor=SeaFloorConfig(albedo=0.2),
        sea_surface=SeaSurfaceConfig(albedo=0.1, roughness=float(np.sqrt(0.05))),
        heatmap=HeatmapConfig(enabled=heatmap, bins=20, water_extent=1.0, seafloor_extent=3.0),
    )


def two_layer_config():
    return SimulationConfig(
        photon_mapping_k=24,
        scene=SceneConfig(flying_height=8.0),
        water=WaterConfig(
            layers=(
                TurbidityLayerConfig(
                    height=0.7, absorption_coefficient=0.2, scattering_coefficient=1.5
                ),
                TurbidityLayerConfig(
                    height=1.3,
                    absorption_coefficient=0.05,
                    scattering_coefficient=0.6,
                    refractive_index=1.36,
                ),
            )
        ),
        laser=LaserConfig(divergence_angle=4e-3, nadir_angle=0.0, pulse_fwhm=3e-9),
        sensor=SensorConfig(aperture_radius=0.05, field_of_view=40e-3, sample_rate=int(1e9)),
        sea_floor=SeaFloorConfig(albedo=0.3),
        heatmap=HeatmapConfig(enabled=False),
    )


def config0_geometry():
    return SimulationConfig(
        scene=SceneConfig(flying_height=400.0),
        water=WaterConfig(
            layers=(
                TurbidityLayerConfig(
                    height=5.0,
                    absorption_coefficient=0.05,
                    scattering_coefficient=0.20,
                    refractive_index=1.34,
                ),
            )
        ),
        laser=LaserConfig(divergence_angle=1e-3, nadir_angle=0.0, pulse_fwhm=3e-9),
        sensor=SensorConfig(field_of_view=20e-3, sample_rate=int(1e10)),
        sea_floor=SeaFloorConfig(albedo=0.15),
        sea_surface=SeaSurfaceConfig(roughness=float(np.sqrt(0.05))),
        heatmap=HeatmapConfig(enabled=False),
    )


def config1_geometry():
    """The large single-instance scene at parity size: 400 m, 20 m water (a 0.10, b 0.40, FF),
    GGX alpha 0.10, albedo 0.20, FOV 50 mrad, 2e10 Hz (0.05 ns bins)."""
    return SimulationConfig(
        scene=SceneConfig(flying_height=400.0),
        water=WaterConfig(
            layers=(
                TurbidityLayerConfig(
                    height=20.0,
                    absorption_coefficient=0.10,
                    scattering_coefficient=0.40,
                    refractive_index=1.34,
                ),
            )
        ),
        laser=LaserConfig(divergence_angle=1e-3, nadir_angle=0.0, pulse_fwhm=3e-9),
        sensor=SensorConfig(field_of_view=50e-3, sample_rate=int(2e10)),
        sea_floor=SeaFloorConfig(albedo=0.20),
        sea_surface=SeaSurfaceConfig(roughness=float(np.sqrt(0.10))),
        heatmap=HeatmapConfig(enabled=False),
    )


def profiled_config():
    """Two depth-profiled layers: linear IOPs and index, then exponential ones with a
    linear salinity profile (TurbidityLayerModel's attenuation LUT, per-step speed)."""
    return SimulationConfig(
        photon_mapping_k=32,
        scene=SceneConfig(flying_height=10.0),
        water=WaterConfig(
            layers=(
                TurbidityLayerConfig(
                    height=1.0,
                    absorption_coefficient=LinearParameter(0.05, 0.3),
                    scattering_coefficient=LinearParameter(0.5, 1.5),
                    refractive_index=LinearParameter(1.33, 1.35),
                ),
                TurbidityLayerConfig(
                    height=1.5,
                    absorption_coefficient=ExponentialParameter(0.1, 0.4),
                    scattering_coefficient=0.8,
                    refractive_index=ExponentialParameter(1.34, 1.36),
                    salinity=LinearParameter(30.0, 38.0),
                ),
            )
        ),
        laser=LaserConfig(divergence_angle=5e-3, nadir_angle=10.0, azimuth_angle=30.0, pulse_fwhm=3e-9),
        sensor=SensorConfig(aperture_radius=0.1, field_of_view=50e-3, sample_rate=int(1e9)),
        sea_floor=SeaFloorConfig(albedo=0.2),
        sea_surface=SeaSurfaceConfig(albedo=0.1, roughness=float(np.sqrt(0.05))),
        heatmap=HeatmapConfig(enabled=False),
    )


def make_replay(only=None):
    jobs = [
        ("small", small_config(), 1500, 400, 11),
        ("twolayer", two_layer_config(), 800, 200, 12),
        ("cfg0", config0_geometry(), 300, 60, 0),
        ("profiled", profiled_config(), 1200, 300, 13),
        ("cfg1", config1_geometry(), 250, 60, 1),
    ]
    if only:
        jobs = [j for j in jobs if j[0] in only]
    for name, cfg, nf, nb, seed in jobs:
        t = time.time()
        out = run_recorded(cfg, nf, nb, seed)
        np.savez_compressed(os.path.join(OUT_DIR, f"replay_{name}.npz"), **out)
        print(f"replay_{name}: {time.time() - t:.1f}s, queries {len(out['queries'])}")


def make_fd_ref():
    """Central differences of the reference simulator itself, for the adjoint columns.

    The 'small' (10 degrees off nadir) and 'cfg0' (nadir: the surface return is gathered at
    the GGX specular peak) replay scenes and seeds, run at seafloor albedo +- 1% and surface
    roughness +- 0.1%. Neither parameter moves a photon or changes how many variates a step
    draws (the albedo scales energies, the roughness only the surface-reflection gather
    weight), so with the same seed each pair replays the base run's variates: a
    common-random-number difference. The generator checks that by comparing the recorded
    streams with the base fixture's. Waveforms are the float64 accumulation of the
    reference's own contributions."""
    import dataclasses

    out = {}
    for job, cfg, nf, nb, seed in (("small", small_config(), 1500, 400, 11),
                                   ("cfg0", config0_geometry(), 300, 60, 0)):
        base = np.load(os.path.join(OUT_DIR, f"replay_{job}.npz"))
        assert int(base["seed"]) == seed and int(base["n_fwd"]) == nf and int(base["n_bwd"]) == nb
        alb = cfg.sea_floor.albedo
        rough = cfg.sea_surface.roughness
        h_alb, h_rough = 0.01 * alb, 1e-3 * rough
        out[f"{job}_h_albedo"] = h_alb
        out[f"{job}_h_roughness"] = h_rough
        floor, surf = cfg.sea_floor, cfg.sea_surface
        runs = (
            ("albedo_plus", dataclasses.replace(cfg, sea_floor=dataclasses.replace(floor, albedo=alb + h_alb))),
            ("albedo_minus", dataclasses.replace(cfg, sea_floor=dataclasses.replace(floor, albedo=alb - h_alb))),
            ("roughness_plus", dataclasses.replace(cfg, sea_surface=dataclasses.replace(surf, roughness=rough + h_rough))),
            ("roughness_minus",
             dataclasses.replace(cfg, sea_surface=dataclasses.replace(surf, roughness=rough - h_rough))),
        )
        for name, c in runs:
            t = time.time()
            r = run_recorded(c, nf, nb, seed)
            for p in ("fwd", "bwd"):
                assert np.array_equal(r[f"{p}_stream"], base[f"{p}_stream"]), (job, name, p, "variates differ")
            out[f"{job}_{name}_waveform64"] = r["waveform64"]
            print(f"fd_ref {job} {name}: {time.time() - t:.1f}s")
    np.savez_compressed(os.path.join(OUT_DIR, "fd_ref.npz"), **out)


def make_kat():
    from alb_sim.math.direction_cone import sample_directions_in_cone_uniform  # noqa: F401
    from alb_sim.math.rotation_matrix import rotation_from_z_batch
    from alb_sim.physics.models.simulation import SimulationModel
    from alb_sim.physics.reflection.fresnel import fresnel_schlick
    from alb_sim.physics.reflection.microfacet_brdf import microfacet_reflected_energy
    from alb_sim.physics.reflection.snell_refraction import calculate_refraction_direction
    from alb_sim.physics.scatter.energy import calculate_energy_batch
    from alb_sim.physics.scatter.fournier_forand_phase_function import (
        calculate_backscatter_fraction,
        calculate_phase_function,
    )

    rng = np.random.default_rng(123)
    out = {}
    ff = [(3.62, 1.1), (3.4, 1.05), (3.9, 1.2)]
    for i, (j, n) in enumerate(ff):
        th, pf, cdf = calculate_phase_function(j, n)
        out[f"ff{i}_params"] = np.array([j, n])
        stride = 1 if i == 0 else 9  # one full table, two subsampled ones
        out[f"ff{i}_stride"] = stride
        out[f"ff{i}_pf"] = pf[::stride]
        out[f"ff{i}_cdf"] = cdf[::stride]
        out[f"ff{i}_bb"] = calculate_backscatter_fraction(j, n)
    # model scalars for several configurations
    cfgs = [small_config(), two_layer_config(), config0_geometry(), SimulationConfig()]
    rows = []
    for cfg in cfgs:
        m = SimulationModel(cfg)
        for li, layer in enumerate(m.water.layers):
            rows.append(
                [
                    cfgs.index(cfg),
                    li,
                    m.steps,
                    m.time_step,
                    m.water_surface_y,
                    m.seafloor_y,
                    layer.lidar_attenuation_coefficient_at(0.0),
                    layer.single_scattering_albedo_at(0.0),
                    layer.light_speed_at(0.0),
                    m.sea_surface.base_reflectance,
                    *m.laser.direction,
                    *m.water_surface_intersection,
                    *m.sea_floor_intersection,
                ]
            )
    out["model_rows"] = np.array(rows, dtype=np.float64)
    # Schlick
    cos = rng.uniform(-0.2, 1.0, 64)
    out["schlick_cos"] = cos
    out["schlick_val"] = fresnel_schlick(cos, 0.0211)
    # Snell (n1=1, n2=1.34) with unit and non-unit incoming directions, both normals
    d = rng.normal(size=(64, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d *= rng.uniform(0.99, 1.01, (64, 1))
    for sgn in (1, -1):
        normal = np.array([0, sgn, 0])
        t, tir = calculate_refraction_direction(d, normal, 1, 1.34)
        out[f"snell_in_{'up' if sgn > 0 else 'down'}"] = d
        out[f"snell_out_{'up' if sgn > 0 else 'down'}"] = t
        out[f"snell_tir_{'up' if sgn > 0 else 'down'}"] = tir
    # rotation matrices including near +z / -z
    v = rng.normal(size=(64, 3))
    v[0] = [0, 0, 1]
    v[1] = [0, 0, -1]
    v[2] = [1e-3, 0, 1]
    v[3] = [0, 2e-3, -1]
    out["rot_in"] = v
    out["rot_out"] = rotation_from_z_batch(v)
    # GGX reflected energy: wi batch, single wo
    wi = rng.normal(size=(256, 3))
    wi[:, 1] = np.abs(wi[:, 1])
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    wo_list = [np.array([0.05, 1.0, -0.02]), np.array([0.3, 0.9, 0.1]), np.array([0.0, -1.0, 0.0])]
    for r_i, rough in enumerate((np.sqrt(0.05), np.sqrt(0.1), 0.5)):
        for w_i, wo in enumerate(wo_list):
            out[f"ggx_{r_i}_{w_i}"] = microfacet_reflected_energy(wi, wo, np.array([0, 1, 0]), rough, 0.0211)
    out["ggx_wi"] = wi
    out["ggx_wo"] = np.array(wo_list)
    out["ggx_rough"] = np.array([np.sqrt(0.05), np.sqrt(0.1), 0.5])
    # scatter energy (bin CDF mass)
    th, pf, cdf = calculate_phase_function(3.62, 1.1)
    pdirs = rng.normal(size=(512, 3)).astype(np.float32)
    pdirs /= np.linalg.norm(pdirs, axis=1, keepdims=True)
    sdir = np.array([0.1, 0.9, -0.2])
    out["senergy_pdirs"] = pdirs
    out["senergy_sdir"] = sdir
    out["senergy_val"] = calculate_energy_batch(pdirs, sdir, th, cdf)
    np.savez_compressed(os.path.join(OUT_DIR, "kat_physics.npz"), **out)
    print("kat_physics written")


def make_knn():
    from scipy.spatial import KDTree

    rng = np.random.default_rng(7)
    out = {}
    # planar disk cluster (surface-like), y fixed
    n = 6000
    r = 0.4 * np.sqrt(rng.random(n))
    ph = rng.uniform(0, 2 * np.pi, n)
    planar = np.stack([r * np.cos(ph), np.full(n, -400.0), r * np.sin(ph)], 1).astype(np.float32)
    # 3-D cloud: dense core and sparse halo
    m = 8000
    core = rng.normal(scale=[0.2, 0.8, 0.2], size=(m // 2, 3)) + [0, -402, 0]
    halo = rng.uniform([-3, -405, -3], [3, -400, 3], size=(m // 2, 3))
    cloud = np.concatenate([core, halo]).astype(np.float32)
    for name, pts, k in (("planar", planar, 100), ("cloud", cloud, 100), ("cloud_k16", cloud, 16)):
        lo, hi = pts.min(0).astype(np.float64), pts.max(0).astype(np.float64)
        span = hi - lo
        near = rng.uniform(lo, hi, size=(300, 3))
        far = rng.uniform(lo - 3 * span - 1, hi + 3 * span + 1, size=(100, 3))
        if name == "planar":
            near[:, 1] = -400.0
            far[:, 1] = -400.0 + rng.normal(scale=1e-9, size=100)
        q = np.concatenate([near, far])
        dist, idx = KDTree(pts).query(q, k=k)
        out[f"{name}_points"] = pts
        out[f"{name}_queries"] = q
        out[f"{name}_idx"] = idx.astype(np.int32)
        out[f"{name}_dist"] = dist
        out[f"{name}_k"] = k
    np.savez_compressed(os.path.join(OUT_DIR, "knn.npz"), **out)
    print("knn written")


def _stats_worker(args):
    seed, nf, nb = args
    from alb_sim.core.simulation import Simulation

    cfg = small_config(heatmap=False)
    sim = Simulation(cfg, np.random.default_rng(seed))
    sim.simulate_batch(nf, forward=True)
    maps = build_photon_map_data(sim.photon_storage)
    for t, data in maps.items():
        sim.photon_maps[t] = PhotonMapIndex(data)
    sim.simulate_batch(nb, forward=False)
    return np.stack([sim.return_waveform[t] for t in TYPES]).astype(np.float64)


def make_stats(runs=32, nf=3000, nb=750):
    with multiprocessing.get_context("spawn").Pool(os.cpu_count()) as pool:
        waves = pool.map(_stats_worker, [(1000 + r, nf, nb) for r in range(runs)])
    w = np.stack(waves) / (nf * nb)  # reference units scale with N_f * N_b
    np.savez_compressed(
        os.path.join(OUT_DIR, "stats_small.npz"),
        mean=w.mean(0),
        se=w.std(0, ddof=1) / np.sqrt(runs),
        per_run=w,
        runs=runs,
        n_fwd=nf,
        n_bwd=nb,
        **config_fields(small_config(heatmap=False)),
    )
    print("stats written")


def _stats_cfg0_worker(args):
    seed, nf, nb = args
    import contextlib
    import io

    from alb_sim.config.run import RunConfig
    from alb_sim.execution.linear import run_linear

    rc = RunConfig(photons_per_batch_forward=nf, photons_per_batch_backward=nb, batches_forward=1,
                   batches_backward=1)
    with contextlib.redirect_stdout(io.StringIO()):
        w = run_linear(config0_geometry(), rc, rng=np.random.default_rng(seed))
    return np.stack([w[t] for t in TYPES]).astype(np.float64)


def make_stats_cfg0(runs=32, nf=8000, nb=2000):
    """Independent runs of the reference's own ``run_linear`` at the config-0 geometry
    (seeds 0 .. runs-1, one forward and one backward batch each). Only the window of bins
    that any run populates is stored (as float32, the reference's waveform type)."""
    with multiprocessing.get_context("spawn").Pool(os.cpu_count()) as pool:
        waves = pool.map(_stats_cfg0_worker, [(r, nf, nb) for r in range(runs)])
    w = np.stack(waves)
    nz = np.nonzero(np.any(w != 0, axis=(0, 1)))[0]
    lo, hi = int(nz[0]), int(nz[-1]) + 1
    w = w[:, :, lo:hi] / (nf * nb)  # reference units scale with N_f * N_b
    np.savez_compressed(
        os.path.join(OUT_DIR, "stats_cfg0.npz"),
        mean=w.mean(0),
        se=w.std(0, ddof=1) / np.sqrt(runs),
        per_run=w.astype(np.float32),
        bin0=lo,
        nbins=int(np.shape(waves[0])[1]),
        runs=runs,
        n_fwd=nf,
        n_bwd=nb,
        **config_fields(config0_geometry()),
    )
    print("stats_cfg0 written", lo, hi)


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    if what in ("kat", "all"):
        make_kat()
    if what in ("knn", "all"):
        make_knn()
    if what in ("replay", "all"):
        make_replay()
    if what == "replay_profiled":
        make_replay(only=("profiled",))
    if what == "replay_cfg1":
        make_replay(only=("cfg1",))
    if what in ("fd_ref", "all"):
        make_fd_ref()
    if what in ("stats", "all"):
        make_stats()
    if what in ("stats_cfg0", "all"):
        make_stats_cfg0()
