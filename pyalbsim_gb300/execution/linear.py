"""Drop-in ``run_linear`` (alb_sim/execution/linear.py:77-117) on the GPU engine.

Same signature, arguments and return value as the reference: a dict mapping each
PhotonType to its float32 return waveform of 2 * steps samples, in the reference's
(unnormalised) units. The forward photons of all batches are traced first, the photon maps
are built once, then the backward photons of all batches are traced and gathered.
"""

from __future__ import annotations

from time import perf_counter
from typing import Optional

import numpy as np

from pyalbsim_gb300.engine import GpuEngine, seed_from_rng


def _report(label, i, batches, t0, t_batch):
    since = perf_counter() - t0
    eta = since / (i + 1) * (batches - (i + 1))
    print(
        f"{label} batch {i + 1}/{batches} in {t_batch:.2f} s = {t_batch / 60:.2f} min, "
        f"{since / 60:.2f} min since start, ETA: {eta / 60:.2f} min"
    )


def linear_forward(engine: GpuEngine, photons_per_batch: int, batches: int, seed: int):
    print("Starting forwards pass")
    t0 = perf_counter()
    for i in range(batches):
        tb = perf_counter()
        engine.forward(photons_per_batch, seed)
        _report("forward", i, batches, t0, perf_counter() - tb)
    print("Finished forwards pass")


def linear_backward(engine: GpuEngine, photons_per_batch: int, batches: int, seed: int):
    print("Starting backwards pass")
    t0 = perf_counter()
    for i in range(batches):
        tb = perf_counter()
        engine.backward(photons_per_batch, seed)
        _report("backward", i, batches, t0, perf_counter() - tb)
    print("Finished backwards pass")


def run_linear(simulation_config, run_config, rng: Optional[np.random.Generator] = None):
    """Forward pass, photon maps, backward pass; returns {PhotonType: float32 waveform}."""
    seed = seed_from_rng(rng)
    engine = GpuEngine(simulation_config)
    try:
        linear_forward(engine, run_config.photons_per_batch_forward, run_config.batches_forward, seed)
        engine.build_maps()
        linear_backward(engine, run_config.photons_per_batch_backward, run_config.batches_backward, seed)
        return engine.waveform(enum_cls=_photon_type_enum(simulation_config))
    finally:
        engine.close()


def _photon_type_enum(simulation_config):
    """Return the reference's PhotonType when the caller passed the reference's config
    objects (so results index the same way), otherwise ours."""
    mod = type(simulation_config).__module__
    if mod.startswith("alb_sim."):
        try:
            from alb_sim.photon_mapping.photon_type import PhotonType as RefPhotonType

            return RefPhotonType
        except ImportError:
            pass
    from pyalbsim_gb300.photon_mapping.photon_type import PhotonType

    return PhotonType
