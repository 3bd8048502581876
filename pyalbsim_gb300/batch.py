"""Batched instances (extension: the reference runs one configuration per call; its
Latin-hypercube notebook loops ``run_parallel`` over the samples).

``hypercube_instances`` draws a sweep as the hypercube notebook does: ``qmc.LatinHypercube``
over depth, a, b, g, albedo, GGX alpha and field of view, with photons per instance
log-uniform over a range (uneven work). ``run_batch`` runs every instance through
``alb_batch_run``: host workers, each owning a device context on its own CUDA stream, take
instances from one queue, largest first, so that small instances overlap on the GPU.
``tune_streams`` is the autotuner. It times the batch on a pilot subset for each candidate
worker count and keeps the fastest. ``run_hypercube`` is the reference's own sweep (seven
config fields, ``run_config`` photon counts) as one batched call.
"""

from __future__ import annotations

import dataclasses
import math
import time
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from pyalbsim_gb300._native import batch_run
from pyalbsim_gb300.adjoint import with_parameters
from pyalbsim_gb300.scene import build_scene

# Sweep ranges: depth (m), a (1/m), b (1/m), HG g, seafloor albedo, GGX alpha, FOV (rad)
RANGES: Dict[str, Tuple[float, float]] = {
    "depth": (1.0, 40.0),
    "absorption": (0.02, 0.5),
    "scattering": (0.05, 1.5),
    "asymmetry": (0.80, 0.95),
    "seafloor_albedo": (0.05, 0.40),
    "ggx_alpha": (0.01, 0.30),
    "field_of_view": (10e-3, 60e-3),
}

LIGHT_SPEED_AIR = 2.998e8


@dataclasses.dataclass
class Instance:
    config: object
    n_forward: int
    n_backward: int
    seed: int
    params: np.ndarray  # depth, a, b, g, albedo, GGX alpha, FOV


def surface_gate(cfg, before: float = 10e-9, length: float = 200e-9) -> Tuple[float, float]:
    """A gate opening ``before`` seconds ahead of the nadir surface return (2 H / c)."""
    t_surface = 2.0 * float(cfg.scene.flying_height) / LIGHT_SPEED_AIR
    return (max(0.0, t_surface - before), length)


def hypercube_instances(
    base_cfg,
    n: int,
    seed: int = 2,
    photons: Tuple[float, float] = (1e5, 1e7),
    backward_fraction: float = 0.25,
    gate: Optional[Tuple[float, float]] = None,
) -> List[Instance]:
    """n instances at ``LatinHypercube(d=7, seed)`` points over RANGES. ``base_cfg`` must have
    one HG water layer; photons per instance are log-uniform over ``photons`` from the same
    seed's stream; Philox seeds are ``seed * 2^32 + i``. ``gate`` (start, length) in seconds
    is applied to every instance."""
    from scipy.stats import qmc

    u = qmc.LatinHypercube(d=7, seed=seed).random(n)
    lo = np.array([r[0] for r in RANGES.values()])
    hi = np.array([r[1] for r in RANGES.values()])
    pts = lo + u * (hi - lo)
    rng = np.random.default_rng(seed)
    nph = np.power(10.0, rng.uniform(math.log10(photons[0]), math.log10(photons[1]), n)).astype(np.int64)
    out = []
    for i in range(n):
        depth, a, b, g, alb, ggx_alpha, fov = pts[i]
        cfg = with_parameters(base_cfg, [depth, a, b, g, alb, math.sqrt(ggx_alpha)])
        cfg = dataclasses.replace(cfg, sensor=dataclasses.replace(cfg.sensor, field_of_view=float(fov)))
        if gate is not None:
            cfg = dataclasses.replace(cfg, waveform_gate=tuple(gate))
        nf = int(nph[i])
        out.append(Instance(cfg, nf, max(1, int(nf * backward_fraction)), (seed << 32) + i, pts[i]))
    return out


def run_batch(instances: Sequence[Instance], streams: int = 8, adjoint: bool = False, precise: bool = False,
              device: int = 0, jacobian_mask: Optional[Sequence[bool]] = None):
    """Every instance through alb_batch_run. Returns (waveforms, jacobians or None,
    statuses, per-instance device ms, wall seconds). With adjoint, ``jacobian_mask`` picks
    the instances that need a Jacobian; the rest run plain."""
    scenes = [build_scene(x.config) for x in instances]
    t0 = time.perf_counter()
    w, j, st, ms = batch_run(
        scenes, [x.n_forward for x in instances], [x.n_backward for x in instances],
        [x.seed for x in instances], streams=streams, precise=precise, adjoint=adjoint, device=device,
        jacobian_mask=jacobian_mask,
    )
    return w, j, st, ms, time.perf_counter() - t0


def tune_streams(
    instances: Sequence[Instance],
    candidates: Sequence[int] = (1, 2, 4, 8, 16),
    pilot: int = 32,
    adjoint: bool = False,
    runner=None,
) -> Tuple[int, Dict[int, float]]:
    """Autotuner: time a pilot subset (every len/pilot-th instance, so its size mix follows
    the batch's) with each candidate worker count and return the fastest and the timings
    (photons per wall second). ``runner(subset, streams) -> wall seconds`` replaces the GPU
    run in tests."""
    step = max(1, len(instances) // max(1, pilot))
    sub = list(instances[::step])[:pilot]
    photons = sum(x.n_forward + x.n_backward for x in sub)
    rates = {}
    for k in candidates:
        if runner is not None:
            wall = runner(sub, k)
        else:
            wall = run_batch(sub, streams=k, adjoint=adjoint)[4]
        rates[k] = photons / wall
    best = max(rates, key=rates.get)
    return best, rates


# The reference's own sweep (its hypercube notebook) varies seven SimulationConfig fields;
# these names select them (plus "asymmetry", the HG extension).
SWEEP_FIELDS = ("height", "absorption", "scattering", "floor_albedo", "surface_roughness",
                "field_of_view", "aperture_radius", "asymmetry")


def config_from_sample(params: Dict[str, float], base=None):
    """A SimulationConfig with the sampled fields set on ``base`` (default: the defaults of
    SimulationConfig) and one water layer; unknown names raise ValueError."""
    from pyalbsim_gb300.config import SimulationConfig, TurbidityLayerConfig, WaterConfig

    unknown = set(params) - set(SWEEP_FIELDS)
    if unknown:
        raise ValueError(f"unknown sweep fields: {sorted(unknown)}")
    cfg = base if base is not None else SimulationConfig()
    layer = cfg.water.layers[0] if base is not None else TurbidityLayerConfig()
    lk = {}
    if "height" in params:
        lk["height"] = float(params["height"])
    if "absorption" in params:
        lk["absorption_coefficient"] = float(params["absorption"])
    if "scattering" in params:
        lk["scattering_coefficient"] = float(params["scattering"])
    if "asymmetry" in params:
        lk["henyey_greenstein_g"] = float(params["asymmetry"])
    sk = {}
    if "field_of_view" in params:
        sk["field_of_view"] = float(params["field_of_view"])
    if "aperture_radius" in params:
        sk["aperture_radius"] = float(params["aperture_radius"])
    cfg = dataclasses.replace(
        cfg,
        water=WaterConfig(layers=(dataclasses.replace(layer, **lk),)),
        sensor=dataclasses.replace(cfg.sensor, **sk),
    )
    if "floor_albedo" in params:
        cfg = dataclasses.replace(cfg, sea_floor=dataclasses.replace(cfg.sea_floor, albedo=float(params["floor_albedo"])))
    if "surface_roughness" in params:
        cfg = dataclasses.replace(
            cfg, sea_surface=dataclasses.replace(cfg.sea_surface, roughness=float(params["surface_roughness"])))
    return cfg


def run_hypercube(param_ranges: Dict[str, Tuple[float, float]], n_samples: int, run_config, seed: Optional[int] = None,
                  base=None, streams: int = 8, device: int = 0, precise: bool = False) -> List[Dict]:
    """The hypercube sweep in one batched call: n_samples LatinHypercube(d) points scaled to
    ``param_ranges``, each simulated with the run_config's photon counts (forward batches x
    photons per batch, backward likewise) through alb_batch_run. Returns
    [{"params": dict, "waveform": {PhotonType: float32 array}}, ...] in sample order.
    With ``seed`` the samples and every instance's Philox key ((seed << 32) + sample index)
    are reproducible. ``precise`` selects the float64-geometry tracer."""
    import secrets

    from scipy.stats import qmc

    from pyalbsim_gb300.photon_mapping.photon_type import PhotonType

    names = list(param_ranges)
    lo = [param_ranges[k][0] for k in names]
    hi = [param_ranges[k][1] for k in names]
    pts = qmc.scale(qmc.LatinHypercube(d=len(names), seed=seed).random(n=n_samples), lo, hi)
    samples = [dict(zip(names, map(float, row))) for row in pts]
    nf = run_config.batches_forward * run_config.photons_per_batch_forward
    nb = run_config.batches_backward * run_config.photons_per_batch_backward
    inst = []
    for i, p in enumerate(samples):
        key = ((int(seed) & 0xFFFFFFFF) << 32) + i if seed is not None else secrets.randbits(64)
        inst.append(Instance(config_from_sample(p, base), nf, nb, key, np.array(list(p.values()))))
    w, _, st, _, _ = run_batch(inst, streams=streams, device=device, precise=precise)
    out = []
    for i, p in enumerate(samples):
        if st[i] != 0:
            raise RuntimeError(f"sample {i} ({p}) failed with status {int(st[i])}")
        out.append({"params": p, "waveform": {t: w[i][c].astype(np.float32) for c, t in enumerate(PhotonType)}})
    return out
