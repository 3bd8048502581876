"""Helpers shared by the tests: golden-fixture loading and configuration rebuilding."""

from __future__ import annotations

import os

import numpy as np

from pyalbsim_gb300.config import (
    HeatmapConfig,
    LaserConfig,
    SceneConfig,
    SeaFloorConfig,
    SeaSurfaceConfig,
    SensorConfig,
    SimulationConfig,
    TurbidityLayerConfig,
    WaterConfig,
)
from pyalbsim_gb300.config.water import FournierForandConfig
from pyalbsim_gb300.utils.parameter_profile import ExponentialParameter, LinearParameter

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_src():
    """Directory holding the reference's importable ``alb_sim`` package, or None: the
    ``ALB_REFERENCE_SRC`` environment variable when it is set, else the copy installed into
    ``baseline/_ref`` by ``python -m pip install --no-deps --target baseline/_ref <reference>``."""
    env = os.environ.get("ALB_REFERENCE_SRC")
    if env:
        return env if os.path.isdir(os.path.join(env, "alb_sim")) else None
    local = os.path.join(REPO, "baseline", "_ref")
    return local if os.path.isdir(os.path.join(local, "alb_sim")) else None


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def config_from_fixture(d) -> SimulationConfig:
    """Rebuild the SimulationConfig a golden fixture was recorded with."""
    f = lambda k: d[k].item() if np.ndim(d[k]) == 0 else d[k]  # noqa: E731
    nl = len(d["cfg_layer_height"])
    prof = d.get("cfg_layer_prof")
    nsub = d.get("cfg_layer_nsub")

    def prop(i, j, plain):
        if prof is None or int(prof[i][j][0]) == 0:
            return float(plain)
        kind, start, end = prof[i][j]
        return (LinearParameter if int(kind) == 1 else ExponentialParameter)(float(start), float(end))

    layers = tuple(
        TurbidityLayerConfig(
            height=float(d["cfg_layer_height"][i]),
            absorption_coefficient=prop(i, 0, d["cfg_layer_a"][i]),
            scattering_coefficient=prop(i, 1, d["cfg_layer_b"][i]),
            salinity=prop(i, 2, d["cfg_layer_salinity"][i]),
            refractive_index=prop(i, 3, d["cfg_layer_n"][i]),
            fournier_forand_parameters=FournierForandConfig(
                refractive_index_ratio=float(d["cfg_layer_nratio"][i]), junge_slope=float(d["cfg_layer_junge"][i])
            ),
            **({"num_sublayers": int(nsub[i])} if nsub is not None else {}),
        )
        for i in range(nl)
    )
    return SimulationConfig(
        sample_multiplier=int(f("cfg_sample_multiplier")),
        photon_mapping_k=int(f("cfg_k")),
        scene=SceneConfig(flying_height=float(f("cfg_flying_height"))),
        water=WaterConfig(layers=layers),
        laser=LaserConfig(
            divergence_angle=float(f("cfg_divergence")),
            wavelength=float(f("cfg_wavelength")),
            nadir_angle=float(f("cfg_nadir")),
            azimuth_angle=float(f("cfg_azimuth")),
            pulse_fwhm=float(f("cfg_pulse_fwhm")),
        ),
        sensor=SensorConfig(
            aperture_radius=float(f("cfg_aperture")),
            field_of_view=float(f("cfg_fov")),
            sample_rate=int(f("cfg_sample_rate")),
        ),
        sea_floor=SeaFloorConfig(albedo=float(f("cfg_floor_albedo"))),
        sea_surface=SeaSurfaceConfig(albedo=float(f("cfg_surface_albedo")), roughness=float(f("cfg_roughness"))),
        heatmap=HeatmapConfig(
            enabled=bool(f("cfg_heatmap_enabled")),
            bins=int(f("cfg_heatmap_bins")),
            water_extent=float(f("cfg_heatmap_water_extent")),
            seafloor_extent=float(f("cfg_heatmap_seafloor_extent")),
        ),
    )


def replay_streams(d, prefix):
    return d[f"{prefix}_offsets"], d[f"{prefix}_stream"], d[f"{prefix}_stream_tau"]


def sort_records(pos, photon, time):
    """Canonical record order: (photon id, time, x, y, z)."""
    return np.lexsort((pos[:, 2], pos[:, 1], pos[:, 0], time, photon))


def assert_statistically_equal(w, st, family_alpha=1e-3):
    """w: [runs, 4, bins] N_f*N_b-normalised waveforms of independent runs; st: the
    reference's per-run waveforms (``per_run``), mean and standard error per bin.

    Two checks per populated bin:
    * CLT regime (both relative standard errors below 25%): |mean - ref| within
      3 combined standard errors; at most the normal tail (plus one bin) may exceed it;
    * every bin, including heavy-tailed ones where a handful of near-spot gathers with
      a tiny k-NN radius dominate a run: a two-sided Mann-Whitney rank test of the
      per-run values must not reject at the family-wise level ``family_alpha``
      (Bonferroni over the tested bins).
    """
    from scipy.stats import mannwhitneyu

    runs = w.shape[0]
    mean, se = w.mean(0), w.std(0, ddof=1) / np.sqrt(runs)
    ref_runs = st["per_run"]
    rmean, rse = st["mean"], st["se"]
    tested = []
    for c in range(4):
        populated = (rmean[c] > 0) | (mean[c] > 0)
        clt = populated & (se[c] < 0.25 * np.abs(mean[c])) & (rse[c] < 0.25 * np.abs(rmean[c]))
        comb = np.sqrt(se[c] ** 2 + rse[c] ** 2)
        z = np.abs(mean[c] - rmean[c])[clt] / comb[clt]
        if z.size:
            assert np.sum(z > 3.0) <= 1 + 0.01 * z.size, (c, np.sort(z)[-5:])
        for b in np.nonzero(populated)[0]:
            a, r = w[:, c, b], ref_runs[:, c, b]
            if np.all(a == a[0]) and np.all(r == a[0]):
                continue
            tested.append((c, b, mannwhitneyu(a, r, alternative="two-sided").pvalue))
    if tested:
        worst = min(tested, key=lambda t: t[2])
        assert worst[2] > family_alpha / len(tested), worst


def per_photon_times(photon, time):
    """{photon id: sorted tuple of its record times}."""
    out = {}
    for p, t in zip(np.asarray(photon).tolist(), np.asarray(time, dtype=np.float64).tolist()):
        out.setdefault(int(p), []).append(t)
    return {p: tuple(sorted(v)) for p, v in out.items()}


def diverged_photons(mine_photon, mine_time, ref_photon, ref_time):
    """Photon ids whose record-time sequences differ between two runs of the same streams."""
    a = per_photon_times(mine_photon, mine_time)
    b = per_photon_times(ref_photon, ref_time)
    return {p for p in set(a) | set(b) if a.get(p) != b.get(p)}


def assert_same_records_except(mine, ref, skip, rtol_pos=1e-5, atol_pos=1e-5):
    """Records of photons not in ``skip``: same ids and times, energies to 1e-6, positions
    to the given tolerance. mine/ref: dicts with photon, time, energy, pos arrays."""
    km = ~np.isin(mine["photon"], list(skip))
    kr = ~np.isin(ref["photon"], list(skip))
    ia = np.lexsort((mine["time"][km], mine["photon"][km]))
    ib = np.lexsort((ref["time"][kr], ref["photon"][kr]))
    np.testing.assert_array_equal(mine["photon"][km][ia], ref["photon"][kr][ib])
    np.testing.assert_array_equal(mine["time"][km][ia], ref["time"][kr][ib])
    np.testing.assert_allclose(mine["energy"][km][ia], ref["energy"][kr][ib], rtol=1e-6)
    np.testing.assert_allclose(mine["pos"][km][ia], ref["pos"][kr][ib], rtol=rtol_pos, atol=atol_pos)
