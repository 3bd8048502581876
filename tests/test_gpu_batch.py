"""Batched instances and gated windows (extensions) on the GPU: the gated waveform is the
slice of the full one, and alb_batch_run over concurrent streams reproduces every
instance's single-instance run bit for bit (waveform and Jacobian). Needs a GB300."""

import dataclasses

import numpy as np
import pytest

from fixtures import config_from_fixture, load
from pyalbsim_gb300 import batch, workloads
from pyalbsim_gb300._native import batch_run
from pyalbsim_gb300.config.gpu import GpuRunOptions
from pyalbsim_gb300.engine import GpuEngine
from pyalbsim_gb300.scene import build_scene

pytestmark = pytest.mark.gpu


def _single(cfg, nf, nb, seed, adjoint=False):
    eng = GpuEngine(cfg, GpuRunOptions(precise=False, adjoint=adjoint))
    try:
        eng.forward(nf, seed)
        eng.build_maps()
        eng.backward(nb, seed)
        return eng.waveform_array(f64=True), (eng.jacobian() if adjoint else None)
    finally:
        eng.close()


@pytest.mark.parametrize("adjoint", [False, True])
def test_gated_waveform_is_the_slice_of_the_full_one(gpu_available, adjoint):
    cfg = dataclasses.replace(config_from_fixture(load("replay_small.npz")))
    full, jf = _single(cfg, 20000, 5000, 4, adjoint)
    sc = build_scene(cfg)
    nz = np.nonzero(full.sum(0))[0]
    width = min(300, full.shape[1] // 3)
    lo = min(int(nz[len(nz) // 3]), full.shape[1] - width - 1)
    gcfg = dataclasses.replace(cfg, waveform_gate=((lo + 0.5) / sc.sample_rate, width / sc.sample_rate))
    g, jg = _single(gcfg, 20000, 5000, 4, adjoint)
    gs = build_scene(gcfg)
    np.testing.assert_array_equal(g, full[:, gs.gate_start:gs.gate_start + gs.n_bins])
    assert g.sum() > 0
    if adjoint:
        np.testing.assert_array_equal(jg, jf[:, :, gs.gate_start:gs.gate_start + gs.n_bins])


def test_gate_with_fixed_radius_stops_early_and_keeps_the_window(gpu_available):
    """Fixed-radius gather: photons stop at the last step that can still reach the window,
    and the window is bit-identical to the full-timeline run's bins."""
    base = workloads.small(0.9, radius=0.5)
    full, _ = _single(base, 50000, 12500, 6)
    gcfg = dataclasses.replace(base, waveform_gate=batch.surface_gate(base))
    gs = build_scene(gcfg)
    g, _ = _single(gcfg, 50000, 12500, 6)
    np.testing.assert_array_equal(g, full[:, gs.gate_start:gs.gate_start + gs.n_bins])
    assert g.sum() > 0


@pytest.mark.parametrize("adjoint,streams", [(False, 4), (True, 3)])
def test_batch_equals_single_instance_runs(gpu_available, adjoint, streams):
    base = workloads.small(0.9, radius=0.5)
    inst = batch.hypercube_instances(base, 12, seed=7, photons=(2e3, 4e4), gate=batch.surface_gate(base))
    w, j, st, ms, wall = batch.run_batch(inst, streams=streams, adjoint=adjoint)
    assert np.all(st == 0), st
    assert np.all(ms > 0)
    for i, x in enumerate(inst):
        ws, js = _single(x.config, x.n_forward, x.n_backward, x.seed, adjoint)
        np.testing.assert_array_equal(w[i], ws)
        if adjoint:
            np.testing.assert_array_equal(j[i], js)
    assert sum(wi.sum() for wi in w) > 0


def test_batch_reports_a_failed_instance_and_runs_the_rest(gpu_available):
    base = workloads.small(0.9, radius=0.5)
    inst = batch.hypercube_instances(base, 4, seed=9, photons=(2e3, 1e4), gate=batch.surface_gate(base))
    scenes = [build_scene(x.config) for x in inst]
    scenes[1].gate_start = 10 ** 9  # a window past the timeline: rejected for this instance only
    w, _, st, _ = batch_run(scenes, [x.n_forward for x in inst], [x.n_backward for x in inst],
                            [x.seed for x in inst], streams=2)
    assert st[1] != 0 and all(st[i] == 0 for i in (0, 2, 3))
    assert not w[1].any() and all(w[i].sum() > 0 for i in (0, 2, 3))


def test_inversion_decreases_the_loss(gpu_available):
    """Adam over the six parameters, every iteration one batch (adjoint + depth pair per
    target): the fixed-key log loss falls."""
    pytest.importorskip("scipy")
    from pyalbsim_gb300 import inversion

    targets = inversion.hypercube_targets(2, seed=4)
    r = inversion.fit(targets, iters=25, lr=2e-2, photons=20000, streams=2)
    h = r["loss_history"]
    assert np.all(np.isfinite(h)) and h[-1] < 0.9 * h[0], h


def test_run_hypercube_matches_single_instance_runs(gpu_available):
    """The reference's sweep as one batched call: every sample equals its own run."""
    pytest.importorskip("scipy")
    from pyalbsim_gb300.config import RunConfig
    from pyalbsim_gb300.config import HeatmapConfig

    ranges = {"height": (0.5, 7.5), "absorption": (0.005, 0.05), "scattering": (1.0, 5.0),
              "floor_albedo": (0.05, 0.3), "surface_roughness": (0.01, 0.1),
              "field_of_view": (5e-3, 40e-3), "aperture_radius": (0.001, 0.2)}
    rc = RunConfig(photons_per_batch_forward=3000, photons_per_batch_backward=1000, batches_forward=2,
                   batches_backward=2)
    base = batch.config_from_sample({}, base=None)
    base = dataclasses.replace(base, heatmap=HeatmapConfig(enabled=False))
    res = batch.run_hypercube(ranges, 4, rc, seed=11, base=base, streams=2)
    assert len(res) == 4
    for i, r in enumerate(res):
        cfg = batch.config_from_sample(r["params"], base)
        key = (11 << 32) + i
        w, _ = _single(cfg, 6000, 2000, key)
        got = np.stack([r["waveform"][t] for t in r["waveform"]])
        np.testing.assert_array_equal(got, w.astype(np.float32))
        assert got.sum() > 0


def test_run_hypercube_samples_match_the_oracle(gpu_available):
    """The sweep driver pinned to the oracle: samples of the reference notebook's seven
    fields, run in one batched call with the float64-geometry tracer, equal the oracle's run
    of the same configuration on the same Philox streams (relative L1 <= 1e-5 per channel)."""
    pytest.importorskip("scipy")
    from oracle.oracle import oracle_run
    from pyalbsim_gb300.config import HeatmapConfig, RunConfig
    from pyalbsim_gb300.scene import build_scene

    ranges = {"height": (0.5, 7.5), "absorption": (0.005, 0.05), "scattering": (1.0, 5.0),
              "floor_albedo": (0.05, 0.3), "surface_roughness": (0.01, 0.1),
              "field_of_view": (5e-3, 40e-3), "aperture_radius": (0.001, 0.2)}
    nf, nb = 1500, 400
    rc = RunConfig(photons_per_batch_forward=nf, photons_per_batch_backward=nb, batches_forward=1,
                   batches_backward=1)
    base = dataclasses.replace(batch.config_from_sample({}, base=None), heatmap=HeatmapConfig(enabled=False))
    res = batch.run_hypercube(ranges, 2, rc, seed=13, base=base, streams=2, precise=True)
    for i, r in enumerate(res):
        cfg = batch.config_from_sample(r["params"], base)
        orc = oracle_run(build_scene(cfg), nf, nb, seed=(13 << 32) + i)["waveform"]
        got = np.stack([r["waveform"][t] for t in r["waveform"]]).astype(np.float64)
        assert orc.sum() > 0
        for c in range(4):
            den = np.abs(orc[c]).sum()
            if den:
                assert np.abs(got[c] - orc[c]).sum() / den < 1e-5, (i, c)


def test_batch_jacobian_mask_runs_masked_instances_plain(gpu_available):
    """With the adjoint on, instances without a Jacobian buffer run plain on the same
    contexts; every waveform still equals its single run."""
    base = workloads.small(0.9, radius=0.5)
    inst = batch.hypercube_instances(base, 6, seed=12, photons=(2e3, 2e4), gate=batch.surface_gate(base))
    mask = [True, False, False, True, False, True]
    w, j, st, _, _ = batch.run_batch(inst, streams=2, adjoint=True, jacobian_mask=mask)
    assert np.all(st == 0), st
    for i, x in enumerate(inst):
        ws, js = _single(x.config, x.n_forward, x.n_backward, x.seed, mask[i])
        np.testing.assert_array_equal(w[i], ws)
        if mask[i]:
            np.testing.assert_array_equal(j[i], js)
        else:
            assert j[i] is None
