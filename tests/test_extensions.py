"""Extensions beyond the reference's own path, on the CPU: the Henyey-Greenstein phase
tables against the closed-form HG CDF and backscatter fraction, and the oracle's
fixed-radius gather against an independent NumPy restatement."""

import dataclasses

import numpy as np
import pytest

from fixtures import config_from_fixture, load
from oracle.oracle import Oracle
from pyalbsim_gb300.config.water import TurbidityLayerConfig
from pyalbsim_gb300.scene import (
    build_scene,
    henyey_greenstein_backscatter,
    henyey_greenstein_table,
)

ALB_BOTTOM_REFLECTION = 0


@pytest.mark.parametrize("g", [0.5, 0.9, 0.95, -0.3])
def test_hg_table_matches_closed_form(g):
    """The running-sum CDF on the phase-table grid follows the closed form
    P(theta) = (1 - g^2) / (2 g) (1 / (1 - g) - 1 / sqrt(1 + g^2 - 2 g cos theta))
    within the grid's quadrature error."""
    th, pf, cdf = henyey_greenstein_table(g)
    exact = (1 - g * g) / (2 * g) * (1 / (1 - g) - 1 / np.sqrt(1 + g * g - 2 * g * np.cos(th)))
    assert np.all(np.diff(cdf) >= 0) and cdf[-1] == 1.0
    assert np.max(np.abs(cdf - exact)) < 2e-3
    # p integrates to one over the sphere
    assert abs(np.trapezoid(2 * np.pi * pf * np.sin(th), th) - 1.0) < 1e-3


@pytest.mark.parametrize("g", [0.5, 0.9, 0.95, -0.3])
def test_hg_backscatter_matches_quadrature(g):
    th = np.linspace(np.pi / 2, np.pi, 200001)
    p = (1 - g * g) / (4 * np.pi * (1 + g * g - 2 * g * np.cos(th)) ** 1.5)
    num = np.trapezoid(2 * np.pi * p * np.sin(th), th)
    assert abs(float(henyey_greenstein_backscatter(g)) - num) < 1e-9


def test_hg_config_validation():
    base = config_from_fixture(load("replay_small.npz")).water.layers[0]
    for bad in (0.0, 1.0, -1.0, 1.5):
        with pytest.raises(ValueError):
            dataclasses.replace(base, henyey_greenstein_g=bad)
    assert isinstance(dataclasses.replace(base, henyey_greenstein_g=0.9), TurbidityLayerConfig)


def test_hg_scene_uses_hg_tables():
    cfg = config_from_fixture(load("replay_small.npz"))
    layers = tuple(dataclasses.replace(L, henyey_greenstein_g=0.9) for L in cfg.water.layers)
    hg = build_scene(dataclasses.replace(cfg, water=dataclasses.replace(cfg.water, layers=layers)))
    ff = build_scene(cfg)
    assert hg.layers[0].backscatter == henyey_greenstein_backscatter(0.9)
    assert hg.layers[0].backscatter != ff.layers[0].backscatter
    assert hg.layers[0].alpha64 != ff.layers[0].alpha64  # Churnside alpha depends on B
    th, _, cdf = henyey_greenstein_table(0.9)
    np.testing.assert_array_equal(hg.layers[0].ff_cdf, cdf)


def test_gather_radius_validation():
    cfg = config_from_fixture(load("replay_small.npz"))
    for bad in (0.0, -0.5):
        with pytest.raises(ValueError):
            dataclasses.replace(cfg, gather_radius=bad)
    assert build_scene(dataclasses.replace(cfg, gather_radius=0.5)).gather_radius == 0.5
    assert build_scene(cfg).gather_radius is None


def _random_map(rng, n, nbins):
    pos = rng.normal(0.0, 0.4, (n, 3)).astype(np.float32)
    pos[:, 1] = np.float32(-10.0)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return dict(
        pos=pos,
        dir=d.astype(np.float32),
        energy=rng.uniform(0.1, 1.0, n).astype(np.float32),
        time=rng.integers(0, nbins * 2, n).astype(np.float32),
    )


def _numpy_radius_gather(scene, m, q, R):
    """Independent restatement: every record with float64 squared distance <= R^2 adds
    (float32(E_q E_p) / (pi R^2)) * albedo / pi * max(0, -d_q.y) to bin
    int(float32(t_q + t_p) / multiplier)."""
    wf = np.zeros(scene.n_bins)
    for i in range(len(q["energy"])):
        d2 = ((m["pos"].astype(np.float64) - q["pos"][i]) ** 2).sum(1)
        sel = d2 <= R * R
        e = (np.float32(q["energy"][i]) * m["energy"][sel]).astype(np.float64)
        w = scene.seafloor_albedo / np.pi * max(0.0, -q["dir"][i][1])
        c = (e * (1.0 / (np.pi * R * R))) * w
        b = ((np.float32(q["time"][i]) + m["time"][sel]) / np.float32(scene.sample_multiplier)).astype(np.int64)
        np.add.at(wf, b, c)
    return wf


def test_oracle_radius_gather_matches_numpy():
    rng = np.random.default_rng(5)
    cfg = config_from_fixture(load("replay_small.npz"))
    R = 0.3
    scene = build_scene(dataclasses.replace(cfg, gather_radius=R))
    m = _random_map(rng, 4000, scene.steps // 2)
    nq = 50
    qd = rng.normal(size=(nq, 3))
    qd /= np.linalg.norm(qd, axis=1, keepdims=True)
    q = dict(
        pos=np.c_[rng.normal(0, 0.4, nq), np.full(nq, -10.0), rng.normal(0, 0.4, nq)],
        dir=qd,
        energy=rng.uniform(0.1, 1.0, nq).astype(np.float32),
        time=rng.integers(0, scene.steps // 2, nq).astype(np.float32),
    )
    wf = np.zeros(scene.n_bins)
    rk = Oracle(scene).gather(ALB_BOTTOM_REFLECTION, m, q, wf)
    np.testing.assert_array_equal(rk, R)
    ref = _numpy_radius_gather(scene, m, q, R)
    np.testing.assert_allclose(wf, ref, rtol=1e-12, atol=1e-300)
    assert ref.sum() > 0


def test_oracle_radius_covering_all_equals_knn_with_k_all():
    """A radius beyond every record admits the whole map, so its estimate is the k = m
    estimate rescaled by r_k^2 / R^2."""
    rng = np.random.default_rng(6)
    cfg = config_from_fixture(load("replay_small.npz"))
    base = build_scene(cfg)
    m = _random_map(rng, 300, base.steps // 2)
    q = dict(pos=np.array([[0.05, -10.0, -0.02]]), dir=np.array([[0.0, -1.0, 0.0]]),
             energy=np.array([0.7], np.float32), time=np.array([3.0], np.float32))
    R = 100.0
    wr = np.zeros(base.n_bins)
    Oracle(build_scene(dataclasses.replace(cfg, gather_radius=R))).gather(ALB_BOTTOM_REFLECTION, m, q, wr)
    wk = np.zeros(base.n_bins)
    rk = Oracle(build_scene(dataclasses.replace(cfg, photon_mapping_k=300))).gather(ALB_BOTTOM_REFLECTION, m, q, wk)
    np.testing.assert_allclose(wr * R * R, wk * rk[0] ** 2, rtol=1e-12)


def test_oracle_radius_gather_on_empty_map_is_zero():
    cfg = config_from_fixture(load("replay_small.npz"))
    scene = build_scene(dataclasses.replace(cfg, gather_radius=0.5))
    m = dict(pos=np.zeros((0, 3), np.float32), dir=np.zeros((0, 3), np.float32),
             energy=np.zeros(0, np.float32), time=np.zeros(0, np.float32))
    q = dict(pos=np.zeros((3, 3)), dir=np.tile([0.0, -1.0, 0.0], (3, 1)),
             energy=np.ones(3, np.float32), time=np.zeros(3, np.float32))
    wf = np.zeros(scene.n_bins)
    Oracle(scene).gather(ALB_BOTTOM_REFLECTION, m, q, wf)
    assert not wf.any()


def _slope_cfg(sigma, name="replay_small.npz"):
    cfg = config_from_fixture(load(name))
    return dataclasses.replace(cfg, sea_surface=dataclasses.replace(cfg.sea_surface, slope_sigma=sigma))


def test_slope_config_validation():
    with pytest.raises(ValueError):
        _slope_cfg(-0.1)
    assert build_scene(_slope_cfg(0.1)).slope_sigma == 0.1
    assert build_scene(_slope_cfg(None)).slope_sigma == 0.0


def test_oracle_slopes_spread_the_refracted_beam():
    """Tilted facets spread the refracted beam: the direction a photon carries into its
    first scatter (the refracted one) varies with the slope std, by about sigma (1 - 1/n)
    per axis, and a zero std is the flat surface exactly."""
    from oracle.oracle import oracle_run

    def first_scatter_dirs(sigma):
        r = oracle_run(build_scene(_slope_cfg(sigma)), 3000, 10, seed=4)
        m = r["maps"][1]
        first = np.unique(m["photon"], return_index=True)[1]
        return r, m["dir"][first]

    flat, dflat = first_scatter_dirs(None)
    zero, _ = first_scatter_dirs(0.0)
    np.testing.assert_array_equal(flat["maps"][0]["pos"], zero["maps"][0]["pos"])
    _, dtilt = first_scatter_dirs(0.2)
    # photons whose first scatter follows a seafloor reflection travel upwards: left out
    dflat, dtilt = dflat[dflat[:, 1] < 0], dtilt[dtilt[:, 1] < 0]
    s_flat, s_tilt = np.std(dflat[:, 2]), np.std(dtilt[:, 2])
    expect = 0.2 * (1 - 1 / 1.33)
    assert s_flat < 0.1 * expect and 0.5 * expect < s_tilt < 2.0 * expect, (s_flat, s_tilt, expect)
