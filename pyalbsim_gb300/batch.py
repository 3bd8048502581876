"""Batched instances (extension: the reference runs one configuration per call; its
Latin-hypercube notebook loops ``run_parallel`` over the samples).

``hypercube_instances`` draws a sweep as the hypercube notebook does: ``qmc.LatinHypercube``
over depth, a, b, g, albedo, GGX alpha and field of view, with photons per instance
log-uniform over a range (uneven work). ``run_batch`` runs every instance through
``alb_batch_run``: host workers, each owning a device context on its own CUDA stream, take
instances from one queue, largest first, so that small instances overlap on the GPU.
``tune_streams`` is the autotuner. It times the batch on a pilot subset for each candidate
worker count and keeps the fastest.
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
              device: int = 0):
    """Every instance through alb_batch_run. Returns (waveforms, jacobians or None,
    statuses, per-instance device ms, wall seconds)."""
    scenes = [build_scene(x.config) for x in instances]
    t0 = time.perf_counter()
    w, j, st, ms = batch_run(
        scenes, [x.n_forward for x in instances], [x.n_backward for x in instances],
        [x.seed for x in instances], streams=streams, precise=precise, adjoint=adjoint, device=device,
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
