"""The oracle's k-d tree neighbour search (its default, used for the CPU baseline) against its
brute-force scan (the checker): the same neighbours in the same order, ties included, and
bit-identical gathers end to end. CPU only."""

import numpy as np
import pytest

from fixtures import config_from_fixture, load
from oracle.oracle import Oracle, oracle_run, set_knn_brute
from pyalbsim_gb300.scene import build_scene


@pytest.fixture
def brute_restored():
    yield
    set_knn_brute(False)


def _both(orc, pts, qs, k):
    set_knn_brute(True)
    a = orc.knn(pts, qs, k)
    set_knn_brute(False)
    b = orc.knn(pts, qs, k)
    return a, b


def _cases(rng):
    cloud = rng.normal(scale=[0.5, 2.0, 0.5], size=(20000, 3)).astype(np.float32)
    planar = np.c_[rng.uniform(-3, 3, 8000), np.full(8000, -5.0), rng.uniform(-3, 3, 8000)].astype(np.float32)
    # exact ties: an integer lattice (many points at equal float64 distances) plus duplicates
    g = np.stack(np.meshgrid(np.arange(12), np.arange(12), np.arange(12)), -1).reshape(-1, 3).astype(np.float32)
    lattice = np.concatenate([g, g[:300]])
    return {"cloud": cloud, "planar": planar, "lattice": lattice}


@pytest.mark.parametrize("k", [1, 7, 100])
def test_tree_knn_equals_brute_force(brute_restored, k):
    rng = np.random.default_rng(5)
    orc = Oracle(build_scene(config_from_fixture(load("replay_small.npz"))), threads=4)
    for name, pts in _cases(rng).items():
        lo, hi = pts.min(0).astype(np.float64), pts.max(0).astype(np.float64)
        qs = np.concatenate([
            rng.uniform(lo - 1.0, hi + 1.0, size=(300, 3)),
            rng.uniform(lo - 50.0, hi + 50.0, size=(50, 3)),   # far queries
            pts[:40].astype(np.float64),                       # queries on map points
            np.round(rng.uniform(lo, hi, size=(60, 3))) + 0.5,  # lattice midpoints: tie-heavy
        ])
        (da, ia), (db, ib) = _both(orc, pts, qs, k)
        np.testing.assert_array_equal(ia, ib, err_msg=name)
        np.testing.assert_array_equal(da, db, err_msg=name)


def test_tree_knn_with_exactly_k_points(brute_restored):
    rng = np.random.default_rng(6)
    orc = Oracle(build_scene(config_from_fixture(load("replay_small.npz"))))
    pts = rng.normal(size=(37, 3)).astype(np.float32)
    qs = rng.normal(size=(20, 3))
    (da, ia), (db, ib) = _both(orc, pts, qs, 37)
    np.testing.assert_array_equal(ia, ib)
    np.testing.assert_array_equal(da, db)


@pytest.mark.parametrize("radius", [None, 0.5])
def test_tree_gather_bit_identical_to_brute_force(brute_restored, radius):
    """k-NN and fixed-radius gathers of a whole run: identical float64 waveforms."""
    import dataclasses

    cfg = config_from_fixture(load("replay_small.npz"))
    if radius is not None:
        cfg = dataclasses.replace(cfg, gather_radius=radius)
    scene = build_scene(cfg)
    set_knn_brute(True)
    a = oracle_run(scene, 3000, 800, seed=77, threads=1)  # one thread: a fixed summation order
    set_knn_brute(False)
    b = oracle_run(scene, 3000, 800, seed=77, threads=1)
    np.testing.assert_array_equal(a["waveform"], b["waveform"])
    for c in a["rk"]:
        np.testing.assert_array_equal(a["rk"][c], b["rk"][c])
    assert a["waveform"].sum() > 0
