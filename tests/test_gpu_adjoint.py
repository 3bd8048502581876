"""Adjoint (extension) on the GPU: record scores and Jacobian against the oracle on the same
Philox streams, the path-independent columns (albedo, roughness) against common-random-
number differences, the score columns (a, b, g) against differences in distribution, the
depth column's return-time shift, and the torch autograd path. Needs a GB300."""

import dataclasses

import numpy as np
import pytest

from fixtures import config_from_fixture, load
from oracle.oracle import oracle_run
from pyalbsim_gb300 import adjoint as adj
from pyalbsim_gb300.config.gpu import GpuRunOptions
from pyalbsim_gb300.engine import GpuEngine
from pyalbsim_gb300.scene import build_scene

pytestmark = pytest.mark.gpu


def _hg_cfg(g=0.9, name="replay_small.npz"):
    cfg = config_from_fixture(load(name))
    layers = tuple(dataclasses.replace(L, henyey_greenstein_g=g) for L in cfg.water.layers)
    return dataclasses.replace(cfg, water=dataclasses.replace(cfg.water, layers=layers))


CFGS = {
    "ff": lambda: config_from_fixture(load("replay_small.npz")),
    "hg": lambda: _hg_cfg(0.9),
    "twolayer": lambda: config_from_fixture(load("replay_twolayer.npz")),
}


def _gpu(cfg, nf, nb, seed, precise=True, adjoint=True, ids=False):
    eng = GpuEngine(cfg, GpuRunOptions(precise=precise, adjoint=adjoint))
    if ids:
        eng.keep_record_ids(True)
    try:
        eng.forward(nf, seed)
        maps = None
        if ids:
            maps = {c: (eng.ctx.export_map(c), eng.ctx.export_map_scores(c)) for c in range(4)}
        eng.build_maps()
        eng.backward(nb, seed)
        w = eng.waveform_array(f64=True)
        j = eng.jacobian() if adjoint else None
    finally:
        eng.close()
    return w, j, maps


@pytest.mark.parametrize("name", list(CFGS))
def test_record_scores_match_oracle(gpu_available, name):
    cfg = CFGS[name]()
    nf, seed = 2000, 11
    _, _, maps = _gpu(cfg, nf, 10, seed, ids=True)
    orc = oracle_run(build_scene(cfg), nf, 10, seed=seed, adjoint=True)
    for c in range(4):
        (pos, dr, e, t, fwi, sfi, pid), sco = maps[c]
        om = orc["maps"][c]
        assert len(e) == len(om["energy"]), c
        ia = np.lexsort((t, pid))
        ib = np.lexsort((om["time"], om["photon"]))
        np.testing.assert_array_equal(pid[ia], om["photon"][ib])
        scale = np.abs(om["score"]).max() + 1.0
        np.testing.assert_allclose(sco[ia], om["score"][ib], rtol=1e-4, atol=1e-5 * scale)


@pytest.mark.parametrize("name", list(CFGS))
def test_jacobian_matches_oracle(gpu_available, name):
    """Same streams, precise tracer: the device Jacobian (float32 scores, fixed-point sums)
    against the oracle's float64 one, per parameter and channel."""
    cfg = CFGS[name]()
    nf, nb, seed = 3000, 800, 21
    w, j, _ = _gpu(cfg, nf, nb, seed)
    orc = oracle_run(build_scene(cfg), nf, nb, seed=seed, adjoint=True)
    oj = orc["jacobian"]
    for p in range(5):
        for c in range(4):
            den = np.abs(oj[p, c]).sum()
            if den == 0:
                assert not j[p, c].any(), (p, c)
                continue
            assert np.abs(j[p, c] - oj[p, c]).sum() / den < 1e-3, (p, c)


def _crn_fd(cfg, field, h, nf, nb, seed):
    p = adj.parameters_of(cfg)
    i = adj.PARAMS.index(field)
    out = []
    for s in (1, -1):
        q = p.copy()
        q[i] += s * h
        w, _, _ = _gpu(adj.with_parameters(cfg, q), nf, nb, seed, precise=False, adjoint=False)
        out.append(w)
    return (out[0] - out[1]) / (2 * h)


@pytest.mark.parametrize("field,col,rel", [("seafloor_albedo", 4, 1e-2), ("roughness", 5, 1e-2)])
def test_path_independent_columns_match_crn_differences(gpu_available, field, col, rel):
    """The albedo and the roughness leave every path unchanged, so with the same streams
    the central difference is smooth and the adjoint column must equal it."""
    cfg = CFGS["hg"]()
    nf, nb, seed = 200000, 50000, 5
    w, j, _ = _gpu(cfg, nf, nb, seed, precise=False)
    h = rel * adj.parameters_of(cfg)[col]
    fd = _crn_fd(cfg, field, h, nf, nb, seed)
    jc = j[col - 1]
    for c in range(4):
        den = np.abs(fd[c]).sum()
        if den > 1e-9 * np.abs(w[c]).sum():
            assert np.abs(jc[c] - fd[c]).sum() / den < 2e-3, c


@pytest.mark.parametrize("field,col", [("absorption", 1), ("scattering", 2), ("asymmetry", 3)])
def test_score_columns_match_differences_in_distribution(gpu_available, field, col):
    """a, b and g move the free paths and scattering angles, so each run's estimate and
    difference are noisy: over 8 seeds the channel-total adjoint derivative agrees with the
    central difference (common random numbers) within 4 combined standard errors plus 2%."""
    cfg = CFGS["hg"]()
    nf, nb = 100000, 25000
    h = 0.05 * adj.parameters_of(cfg)[col]
    J, F = [], []
    for s in range(8):
        _, j, _ = _gpu(cfg, nf, nb, 1000 + s, precise=False)
        J.append(j[col - 1].sum(1))
        F.append(_crn_fd(cfg, field, h, nf, nb, 1000 + s).sum(1))
    J, F = np.array(J), np.array(F)
    se = np.sqrt(J.var(0, ddof=1) / 8 + F.var(0, ddof=1) / 8)
    mj, mf = J.mean(0), F.mean(0)
    assert np.all(np.abs(mj - mf) <= 4 * se + 0.02 * np.abs(mf) + 1e-30), (field, mj, mf, se)


def _centroid_rate(w, jac):
    t = np.arange(w.shape[1]) + 0.5
    W, J = w[0], jac[0, 0]
    return (t * J).sum() / W.sum() - (t * W).sum() * J.sum() / W.sum() ** 2


def test_depth_column_shifts_the_bottom_return(gpu_available):
    """d/d depth of the bottom-channel centroid: both legs lengthen by about one depth step
    each, so the return moves by 2 n / c per metre (in bins of dt * multiplier). Central
    difference, one seed."""
    cfg = CFGS["hg"]()
    scene = build_scene(cfg)
    nf, nb, seed = 200000, 50000, 9
    w, jac = adj.simulate_with_jacobian(cfg, nf, nb, seed, GpuRunOptions(precise=False), depth_step=0.05,
                                        depth_difference="central")
    bin_s = scene.dt * scene.sample_multiplier
    expect = 2.0 / (scene.layers[-1].speed32 * bin_s)
    dcent = _centroid_rate(w, jac)
    assert 0.8 * expect < dcent < 1.3 * expect, (dcent, expect)


def test_forward_depth_column_shifts_the_bottom_return(gpu_available):
    """The default forward difference (one extra run), averaged over six seeds.

    The simulated time span follows the depth (the reference sets its step count from it):
    at this scene it gains a step every ~0.2 m (at 2.05 m, just above the scene's 2 m), and
    a longer span admits late photons, a jump in the waveform that a difference across it
    includes. The depth is therefore set to 1.9 m, whose interval [1.9, 1.95] m keeps one
    span. There the centroid is convex in the depth: small-step differences of the oracle
    (h = 0.01 m, 10 seeds) give 11.8 +- 0.4 bins/m central and 12.2 +- 0.5 forward, against
    the 8.9 bins/m of a pure time shift (the return also changes shape), and 9.8 central at
    h = 0.05 m. The bar is the pure shift's rate times [0.8, 1.6], which holds the measured
    rates and rejects a column of the wrong sign or scale."""
    cfg = CFGS["hg"]()
    p = adj.parameters_of(cfg)
    p[0] = 1.9
    cfg = adj.with_parameters(cfg, p)
    scene = build_scene(cfg)
    assert build_scene(adj.with_parameters(cfg, p + np.array([0.05, 0, 0, 0, 0, 0]))).steps == scene.steps
    nf, nb = 200000, 50000
    rates = []
    for seed in range(20, 26):
        w, jac = adj.simulate_with_jacobian(cfg, nf, nb, seed, GpuRunOptions(precise=False), depth_step=0.05)
        rates.append(_centroid_rate(w, jac))
    bin_s = scene.dt * scene.sample_multiplier
    expect = 2.0 / (scene.layers[-1].speed32 * bin_s)
    assert 0.8 * expect < np.mean(rates) < 1.6 * expect, (rates, expect)


def test_torch_gradient_equals_c_adjoint(gpu_available):
    torch = pytest.importorskip("torch")
    cfg = CFGS["hg"]()
    nf, nb, seed = 20000, 5000, 3
    p = torch.tensor(adj.parameters_of(cfg), dtype=torch.float64, requires_grad=True)
    w = adj.WaveformFunction.apply(p, cfg, nf, nb, seed, GpuRunOptions(precise=False))
    target = torch.zeros_like(w)
    loss = ((w - target) ** 2).sum()
    loss.backward()
    dL = 2.0 * w.detach().numpy()
    eng = GpuEngine(cfg, GpuRunOptions(precise=False, adjoint=True))
    try:
        eng.forward(nf, seed)
        eng.build_maps()
        eng.backward(nb, seed)
        np.testing.assert_array_equal(eng.waveform_array(), w.detach().numpy())
        g = eng.ctx.adjoint(dL)
    finally:
        eng.close()
    assert np.isnan(g[0])
    np.testing.assert_allclose(p.grad.numpy()[1:], g[1:], rtol=1e-9)
    assert np.isfinite(p.grad.numpy()[0]) and p.grad.numpy()[0] != 0.0


@pytest.mark.parametrize("job", ["small", "cfg0"])
def test_columns_match_reference_simulator_differences(gpu_available, job):
    """The GPU's albedo and roughness columns, replaying the reference's own variates,
    against central differences of the reference simulator at the same seed (fixture): 1e-4
    in L1 per reached channel (float32 contributions against the reference's float64 sums)."""
    from fixtures import replay_streams
    from test_adjoint_host import assert_columns_match_reference_differences

    d = load(f"replay_{job}.npz")
    cfg = config_from_fixture(d)
    eng = GpuEngine(cfg, GpuRunOptions(precise=True, adjoint=True))
    try:
        eng.forward(int(d["n_fwd"]), 0, replay=replay_streams(d, "fwd"))
        eng.build_maps()
        eng.backward(int(d["n_bwd"]), 0, replay=replay_streams(d, "bwd"))
        jac = eng.jacobian()
    finally:
        eng.close()
    assert_columns_match_reference_differences(jac, d, job, tol=1e-4)
