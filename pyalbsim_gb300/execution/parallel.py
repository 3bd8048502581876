"""Drop-in ``run_parallel`` (alb_sim/execution/parallel.py:186-284) on the GPU engine.

The reference fans independent batches out to a process pool, merges the photon
storages, rebuilds a KD-tree per worker and sums the worker waveforms and heatmaps. On
one GPU all batches run in one context: the maps are appended batch by batch, built once,
and every backward batch accumulates into the same exact fixed-point waveform, which is
the sum the reference's merge computes.

Seeding follows the reference: with ``seed=None`` every batch draws an independent
stream; with a fixed seed every batch receives THE SAME seed (parallel.py:210-212,
239-242), so all forward batches are identical copies and so are all backward batches.
That behaviour is kept so that seeded results compare with the reference's.
"""

from __future__ import annotations

import secrets
from time import perf_counter
from typing import Optional

from pyalbsim_gb300.engine import GpuEngine
from pyalbsim_gb300.execution.linear import _photon_type_enum


def merge_results(results):
    """Sum per-batch waveform dicts (parallel.py:24-44)."""
    import numpy as np

    merged = {}
    for result in results:
        for photon_type, arr in result.items():
            merged.setdefault(photon_type, []).append(arr)
    return {t: np.sum(a, axis=0) for t, a in merged.items()}


def _map_classes(simulation_config):
    mod = type(simulation_config).__module__
    if mod.startswith("alb_sim."):
        try:
            from alb_sim.photon_mapping.photon_map_data import PhotonMapData
            from alb_sim.utils.heatmap_result import SampledHeatmapsResult

            return PhotonMapData, SampledHeatmapsResult
        except ImportError:
            pass
    from pyalbsim_gb300.photon_mapping.photon_map_data import PhotonMapData
    from pyalbsim_gb300.utils.heatmap_result import SampledHeatmapsResult

    return PhotonMapData, SampledHeatmapsResult


def run_parallel(simulation_config, run_config, seed: Optional[int] = None):
    """Returns (waveform dict, photon_maps_data dict, SampledHeatmapsResult or None)."""
    engine = GpuEngine(simulation_config)
    enum_cls = _photon_type_enum(simulation_config)
    map_cls, heat_cls = _map_classes(simulation_config)
    try:
        print("Starting forwards pass")
        t0 = perf_counter()
        nf = run_config.photons_per_batch_forward
        for i in range(run_config.batches_forward):
            batch_seed = seed if seed is not None else secrets.randbits(64)
            # a fixed seed replays the same photons in every batch, as in the reference
            engine.forward(nf, batch_seed, first=0 if seed is not None else None)
            print(f"forward batch {i + 1}/{run_config.batches_forward} ({perf_counter() - t0:.2f} s since start)")
        engine.build_maps()
        print("Starting backward pass...")
        nb = run_config.photons_per_batch_backward
        for i in range(run_config.batches_backward):
            batch_seed = seed if seed is not None else secrets.randbits(64)
            engine.backward(nb, batch_seed, first=0 if seed is not None else None)
            print(f"backward batch {i + 1}/{run_config.batches_backward} ({perf_counter() - t0:.2f} s since start)")
        waveform = engine.waveform(enum_cls=enum_cls)
        maps = engine.photon_maps_data(enum_cls=enum_cls, data_cls=map_cls)
        heat = engine.heatmaps(result_cls=heat_cls)
        return waveform, maps, heat
    finally:
        engine.close()
