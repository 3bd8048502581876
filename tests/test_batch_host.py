"""Batched instances and gated windows (extensions) on the CPU: the Latin-hypercube sweep,
the worker-count autotuner, and the oracle's gated window against its full timeline."""

import dataclasses

import numpy as np
import pytest

from fixtures import config_from_fixture, load
from oracle.oracle import oracle_run
from pyalbsim_gb300 import batch, workloads
from pyalbsim_gb300.scene import build_scene


def test_hypercube_is_stratified_and_in_range():
    pytest.importorskip("scipy")
    inst = batch.hypercube_instances(workloads.small(0.9), 64, seed=2, photons=(1e5, 1e7))
    P = np.array([x.params for x in inst])
    for j, (lo, hi) in enumerate(batch.RANGES.values()):
        assert np.all((P[:, j] >= lo) & (P[:, j] <= hi))
        strata = np.floor((P[:, j] - lo) / (hi - lo) * 64).astype(int)
        assert len(set(strata.tolist())) == 64  # one point per stratum: Latin hypercube
    nf = np.array([x.n_forward for x in inst])
    assert nf.min() >= 1e5 and nf.max() <= 1e7 and nf.max() / nf.min() > 10
    again = batch.hypercube_instances(workloads.small(0.9), 64, seed=2)
    assert all(a.n_forward == b.n_forward and np.array_equal(a.params, b.params) for a, b in zip(inst, again))
    x = inst[5]
    sc = build_scene(x.config)
    assert abs(sc.depth - x.params[0]) < 1e-9 and abs(sc.fov - x.params[6]) < 1e-12
    assert abs(sc.roughness ** 2 - x.params[5]) < 1e-12 and sc.layers[0].hg_g == pytest.approx(x.params[3])


def test_autotuner_picks_the_fastest_worker_count():
    pytest.importorskip("scipy")
    inst = batch.hypercube_instances(workloads.small(0.9), 40, seed=3, photons=(1e4, 1e5))
    cost = {1: 4.0, 2: 2.5, 4: 1.5, 8: 1.2, 16: 1.6}
    best, rates = batch.tune_streams(inst, pilot=8, runner=lambda sub, k: cost[k])
    assert best == 8 and set(rates) == set(cost)


def test_surface_gate_brackets_the_surface_return():
    cfg = workloads.small(0.9)
    start, length = batch.surface_gate(cfg)
    sc = build_scene(dataclasses.replace(cfg, waveform_gate=(start, length)))
    assert sc.n_bins == round(length * sc.sample_rate)
    t_surf_bin = 2 * 400.0 / 2.998e8 * sc.sample_rate
    assert sc.gate_start < t_surf_bin < sc.gate_start + sc.n_bins


def test_gate_validation():
    cfg = config_from_fixture(load("replay_small.npz"))
    for bad in ((-1e-9, 1e-7), (0.0, 0.0)):
        with pytest.raises(ValueError):
            dataclasses.replace(cfg, waveform_gate=bad)
    with pytest.raises(ValueError):
        build_scene(dataclasses.replace(cfg, waveform_gate=(0.0, 1.0)))  # longer than the timeline


def test_oracle_gated_window_is_a_slice_of_the_timeline():
    cfg = config_from_fixture(load("replay_small.npz"))
    full = oracle_run(build_scene(cfg), 1500, 400, seed=8)["waveform"]
    nz = np.nonzero(full.sum(0))[0]
    width = min(300, full.shape[1] // 3)
    lo = min(int(nz[len(nz) // 3]), full.shape[1] - width - 1)
    rate = build_scene(cfg).sample_rate
    gated_cfg = dataclasses.replace(cfg, waveform_gate=((lo + 0.5) / rate, width / rate))
    sc = build_scene(gated_cfg)
    g = oracle_run(sc, 1500, 400, seed=8)["waveform"]
    assert g.shape == (4, sc.n_bins)
    np.testing.assert_allclose(g, full[:, sc.gate_start:sc.gate_start + sc.n_bins], rtol=1e-12, atol=0)
    assert g.sum() > 0


def test_inversion_targets_follow_the_sweep_ranges():
    pytest.importorskip("scipy")
    from pyalbsim_gb300 import inversion

    t = inversion.hypercube_targets(32, seed=4)
    assert t.shape == (32, 6)
    assert np.all((t[:, 0] >= 1) & (t[:, 0] <= 40)) and np.all((t[:, 3] >= 0.8) & (t[:, 3] <= 0.95))
    assert np.all((t[:, 5] ** 2 >= 0.01) & (t[:, 5] ** 2 <= 0.30))
    sc = build_scene(inversion.gated_base())
    assert sc.n_bins == round(400e-9 * sc.sample_rate)


def test_config_from_sample_sets_the_sweep_fields():
    p = {"height": 3.0, "absorption": 0.02, "scattering": 2.0, "floor_albedo": 0.1,
         "surface_roughness": 0.05, "field_of_view": 0.01, "aperture_radius": 0.05}
    sc = build_scene(batch.config_from_sample(p))
    assert (sc.depth, sc.fov, sc.aperture_radius, sc.seafloor_albedo, sc.roughness) == (3.0, 0.01, 0.05, 0.1, 0.05)
    assert sc.layers[0].absorption == 0.02
    with pytest.raises(ValueError):
        batch.config_from_sample({"depth": 3.0})
