"""The inversion loop on the CPU against an analytic stand-in for the batched simulator:
Adam in log-parameter space, the depth column from each iteration's depth pair, the
Jacobian mask and the coarse depth-grid start recover the parameters of a toy waveform
model whose derivatives are exact."""

import numpy as np
import pytest

from pyalbsim_gb300 import inversion

NB = 600
T = np.arange(NB, dtype=np.float64)


def _toy(theta):
    """Channel 0: seafloor peak (time 20 + 8 depth, height albedo e^(-2 a depth)) + surface
    peak (height ~ roughness) + volume tail (b g). Returns (w [4, NB], d w / d (a, b, g,
    albedo, roughness) [5, 4, NB])."""
    D, a, b, g, alb, r = theta
    peak = np.exp(-((T - 20.0 - 8.0 * D) ** 2) / 50.0)
    surf = np.exp(-((T - 10.0) ** 2) / 8.0)
    tail = np.exp(-T / 50.0)
    att = np.exp(-2.0 * a * D)
    w = np.zeros((4, NB))
    w[0] = alb * att * peak + 3.0 * r * surf + 0.5 * b * g * tail
    j = np.zeros((5, 4, NB))
    j[0, 0] = -2.0 * D * alb * att * peak
    j[1, 0] = 0.5 * g * tail
    j[2, 0] = 0.5 * b * tail
    j[3, 0] = att * peak
    j[4, 0] = 3.0 * surf
    return w * 1e3, j * 1e3


def _fake_run_batch(instances, streams=8, adjoint=False, precise=False, device=0, jacobian_mask=None):
    ws, js = [], []
    for k, x in enumerate(instances):
        w, j = _toy(np.asarray(x.params, dtype=np.float64))
        ws.append(w)
        want = adjoint and (jacobian_mask is None or jacobian_mask[k])
        js.append(j if want else None)
    st = np.zeros(len(instances), np.int32)
    return ws, (js if adjoint else None), st, np.zeros(len(instances)), 0.0


@pytest.fixture
def fake(monkeypatch):
    monkeypatch.setattr(inversion, "run_batch", _fake_run_batch)
    monkeypatch.setattr(inversion, "with_parameters", lambda base, p: None)


@pytest.mark.parametrize("loss", ["mse", "log", "poisson"])
def test_fit_recovers_a_nearby_target(fake, loss):
    target = np.array([[11.0, 0.12, 0.33, 0.88, 0.22, 0.30]])
    r = inversion.fit(target, iters=400, lr=2e-2, photons=100, peak=1e6, base=object(), loss=loss,
                      depth_step=0.05)
    h = r["loss_history"]
    # the log loss keeps the Poisson floor of the many low-count bins
    assert h[-1] < (1e-2 if loss == "mse" else 0.9) * h[0], (h[0], h[-1])
    assert abs(r["depth_error"][0]) < 0.05, r["params"]
    # the toy sees albedo and a only through the peak height, and b and g through b g
    P, Q = r["params"][0], target[0]
    height = lambda x: x[4] * np.exp(-2.0 * x[1] * x[0])  # noqa: E731
    np.testing.assert_allclose([height(P), P[2] * P[3], P[5]], [height(Q), Q[2] * Q[3], Q[5]],
                               rtol=0.03 if loss == "mse" else 0.06)


def test_depth_grid_start_finds_a_distant_seafloor(fake):
    """From 10 m the seafloor peak of a 30 m target does not overlap: without the grid the
    depth has no slope; the grid start lands next to it and the fit closes in."""
    target = np.array([[30.0, 0.10, 0.30, 0.90, 0.20, float(np.sqrt(0.1))]])
    plain = inversion.fit(target, iters=150, lr=2e-2, photons=100, peak=1e6, base=object(), loss="log")
    grid = inversion.fit(target, iters=150, lr=2e-2, photons=100, peak=1e6, base=object(), loss="log",
                         depth_grid=np.linspace(2, 38, 10))
    assert abs(plain["depth_error"][0]) > 5.0
    assert abs(grid["depth_error"][0]) < 0.1, grid["params"]


def test_fixed_parameters_make_attenuation_identifiable(fake):
    """With the albedo and g known (fixed at the truth) the toy separates a from the albedo
    and b from g: a and b are recovered individually, and fixed values do not move."""
    target = np.array([[11.0, 0.12, 0.33, 0.88, 0.22, 0.30]])
    initial = np.array([10.0, 0.10, 0.30, 0.88, 0.22, 0.25])
    r = inversion.fit(target, iters=400, lr=2e-2, photons=100, peak=1e6, base=object(), loss="mse",
                      initial=initial, fixed=[False, False, False, True, True, False])
    P = r["params"][0]
    assert P[3] == initial[3] and P[4] == initial[4]
    np.testing.assert_allclose(P[[0, 1, 2, 5]], target[0, [0, 1, 2, 5]], rtol=0.03)


def test_fixed_depth_skips_the_depth_pair(fake, monkeypatch):
    calls = []

    def counting(instances, **kw):
        calls.append(len(instances))
        return _fake_run_batch(instances, **kw)

    monkeypatch.setattr(inversion, "run_batch", counting)
    target = np.array([[11.0, 0.12, 0.33, 0.88, 0.22, 0.30], [9.0, 0.1, 0.3, 0.9, 0.2, 0.3]])
    inversion.fit(target, iters=3, photons=100, base=object(), fixed=[True] + [False] * 5)
    assert calls == [2, 2, 2, 2]  # the targets, then one adjoint instance per target and iteration
    calls.clear()
    inversion.fit(target, iters=2, photons=100, base=object())
    assert calls == [2, 4, 4]  # forward depth difference: one shifted instance per target
    calls.clear()
    inversion.fit(target, iters=2, photons=100, base=object(), depth_difference="central")
    assert calls == [2, 6, 6]


def test_prior_holds_a_parameter_near_its_start(fake):
    """With the Poisson likelihood, a tight prior on ln(b / b0) keeps b near its start (g
    takes up the product b g the toy sees); a flat one lets b move."""
    target = np.array([[11.0, 0.12, 0.45, 0.88, 0.22, 0.30]])
    kw = dict(iters=300, lr=2e-2, photons=100, peak=1e6, base=object(), loss="poisson")
    flat = inversion.fit(target, **kw)
    tight = inversion.fit(target, prior_sigma=[None, None, 1e-5, None, None, None], **kw)
    b0 = inversion.INITIAL[2]
    assert abs(tight["params"][0, 2] / b0 - 1.0) < 0.05, tight["params"]
    assert abs(flat["params"][0, 2] / b0 - 1.0) > 0.15, flat["params"]
    with pytest.raises(ValueError):
        inversion.fit(target, prior_sigma=[0.0] * 6, **kw)


def _toy_channels(theta):
    """The toy with its seafloor peak alone in channel 0, as the simulator's seafloor
    channel holds it, and the volume tail and surface peak in channels 1 and 2."""
    D, a, b, g, alb, r = theta
    peak = np.exp(-((T - 20.0 - 8.0 * D) ** 2) / 50.0)
    surf = np.exp(-((T - 10.0) ** 2) / 8.0)
    tail = np.exp(-T / 50.0)
    att = np.exp(-2.0 * a * D)
    w = np.zeros((4, NB))
    w[0] = alb * att * peak
    w[1] = 0.5 * b * g * tail
    w[2] = 3.0 * r * surf
    j = np.zeros((5, 4, NB))
    j[0, 0] = -2.0 * D * alb * att * peak
    j[1, 1] = 0.5 * g * tail
    j[2, 1] = 0.5 * b * tail
    j[3, 0] = att * peak
    j[4, 2] = 3.0 * surf
    return w * 1e3, j * 1e3


def _fake_run_batch_channels(instances, streams=8, adjoint=False, precise=False, device=0, jacobian_mask=None):
    ws, js = [], []
    for k, x in enumerate(instances):
        w, j = _toy_channels(np.asarray(x.params, dtype=np.float64))
        ws.append(w)
        js.append(j if adjoint and (jacobian_mask is None or jacobian_mask[k]) else None)
    return ws, (js if adjoint else None), np.zeros(len(instances), np.int32), np.zeros(len(instances)), 0.0


def test_depth_start_from_the_seafloor_peak(monkeypatch):
    """A 30 m target is 20 m from the 10 m start, where the loss has no depth slope: the
    start read from the target's own seafloor peak (calibrated by two model runs) lands
    next to it and the fit closes in. A target with no visible seafloor return keeps its
    start and is reported as undetectable."""
    monkeypatch.setattr(inversion, "run_batch", _fake_run_batch_channels)
    monkeypatch.setattr(inversion, "with_parameters", lambda base, p: None)
    target = np.array([[30.0, 0.10, 0.30, 0.90, 0.20, float(np.sqrt(0.1))],
                       [25.0, 0.10, 0.30, 0.90, 1e-9, float(np.sqrt(0.1))]])
    kw = dict(photons=100, peak=1e6, base=object(), loss="log", depth_init="bottom_peak")
    start = inversion.fit(target, iters=0, **kw)  # the starts themselves
    assert start["depth_detectable"].tolist() == [True, False]
    assert abs(start["depth_error"][0]) < 0.5, start["params"]
    assert start["params"][1, 0] == inversion.INITIAL[0]
    r = inversion.fit(target, iters=150, lr=2e-2, **kw)
    assert abs(r["depth_error"][0]) < 0.1, r["params"]
    with pytest.raises(ValueError):
        inversion.fit(target, iters=1, photons=100, base=object(), depth_init="centroid")


def test_depth_start_without_a_calibration_shift_keeps_every_start(monkeypatch):
    """If the two calibration runs put the seafloor peak in the same bin (no usable depth
    scale), no target's depth start is changed and none is reported detectable."""
    def flat(instances, streams=8, adjoint=False, precise=False, device=0, jacobian_mask=None):
        ws, js = [], []
        for x in instances:
            w, j = _toy_channels(np.asarray(x.params, dtype=np.float64))
            w[0] = 0.0
            w[0, 300] = 1e3  # the same peak bin whatever the depth
            ws.append(w)
            js.append(j if adjoint else None)
        return ws, (js if adjoint else None), np.zeros(len(instances), np.int32), np.zeros(len(instances)), 0.0

    monkeypatch.setattr(inversion, "run_batch", flat)
    monkeypatch.setattr(inversion, "with_parameters", lambda base, p: None)
    target = np.array([[30.0, 0.10, 0.30, 0.90, 0.20, float(np.sqrt(0.1))]])
    r = inversion.fit(target, iters=0, photons=100, peak=1e6, base=object(), depth_init="bottom_peak")
    assert r["depth_detectable"].tolist() == [False]
    assert r["params"][0, 0] == inversion.INITIAL[0]
