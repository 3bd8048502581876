"""Differentiable waveform (extension: the reference has no derivatives).

Parameters, in this order: water depth, absorption a, scattering b, Henyey-Greenstein
asymmetry g, seafloor albedo, surface roughness. a, b and g are set on every water layer
(constant layers only); the depth is the sum of the layer heights and moves the lowest
layer's floor.

Columns a, b, g, albedo and roughness come from the device adjoint (path scores carried by
every record and query, accumulated in the same gather as the waveform). The depth moves
the seafloor plane and with it the discrete integrator step at which a photon returns, so
its column is a difference with common random numbers (the same Philox streams traced at
another depth): by default a forward difference against the adjoint run's own waveform,
one extra run at depth + h (its O(h) bias against the central difference is measured by
``depth_difference_bias``); ``depth_difference="central"`` traces depth +- h instead.

``WaveformFunction`` wraps one simulation as a ``torch.autograd.Function``: forward returns
the float64 waveform [channels, nbins]; backward contracts the incoming gradient with the
Jacobian.
"""

from __future__ import annotations

import dataclasses
from typing import Optional, Sequence, Tuple

import numpy as np

from pyalbsim_gb300.config.gpu import GpuRunOptions
from pyalbsim_gb300.engine import GpuEngine

PARAMS = ("depth", "absorption", "scattering", "asymmetry", "seafloor_albedo", "roughness")


def parameters_of(cfg) -> np.ndarray:
    """The six parameters of a configuration (g = 0 for a Fournier-Forand water column)."""
    layers = cfg.water.layers
    top = layers[0]
    g = getattr(top, "henyey_greenstein_g", None)
    return np.array([
        float(sum(float(L.height) for L in layers)),
        float(top.absorption_coefficient),
        float(top.scattering_coefficient),
        0.0 if g is None else float(g),
        float(cfg.sea_floor.albedo),
        float(cfg.sea_surface.roughness),
    ])


def with_parameters(cfg, params: Sequence[float]):
    """A copy of ``cfg`` with the six parameters applied (g only on HG layers)."""
    depth, a, b, g, albedo, rough = (float(x) for x in params)
    layers = list(cfg.water.layers)
    above = sum(float(L.height) for L in layers[:-1])
    if not depth > above:
        raise ValueError("depth must exceed the height of the layers above the lowest one")
    out = []
    for i, L in enumerate(layers):
        kw = dict(absorption_coefficient=a, scattering_coefficient=b)
        if getattr(L, "henyey_greenstein_g", None) is not None:
            kw["henyey_greenstein_g"] = g
        if i == len(layers) - 1:
            kw["height"] = depth - above
        out.append(dataclasses.replace(L, **kw))
    return dataclasses.replace(
        cfg,
        water=dataclasses.replace(cfg.water, layers=tuple(out)),
        sea_floor=dataclasses.replace(cfg.sea_floor, albedo=albedo),
        sea_surface=dataclasses.replace(cfg.sea_surface, roughness=rough),
    )


def _run(cfg, n_fwd: int, n_bwd: int, seed: int, options: GpuRunOptions, adjoint: bool):
    eng = GpuEngine(cfg, dataclasses.replace(options, adjoint=adjoint))
    try:
        eng.forward(n_fwd, seed)
        eng.build_maps()
        eng.backward(n_bwd, seed)
        w = eng.waveform_array(f64=True)
        j = eng.jacobian() if adjoint else None
    finally:
        eng.close()
    return w, j


def simulate_with_jacobian(
    cfg,
    n_fwd: int,
    n_bwd: int,
    seed: int,
    options: Optional[GpuRunOptions] = None,
    depth_step: Optional[float] = None,
    with_depth: bool = True,
    depth_difference: str = "forward",
) -> Tuple[np.ndarray, np.ndarray]:
    """One simulation: (waveform float64 [4, nbins], Jacobian float64 [6, 4, nbins]).

    depth_step (m): step of the depth difference, default max(1% of the depth, 1 cm).
    depth_difference: "forward" ((w(d + h) - w(d)) / h, one extra run) or "central"
    ((w(d + h) - w(d - h)) / 2h, two extra runs). with_depth=False leaves the depth column
    at zero and skips the extra runs."""
    if depth_difference not in ("forward", "central"):
        raise ValueError("depth_difference must be 'forward' or 'central'")
    options = options or GpuRunOptions()
    w, j5 = _run(cfg, n_fwd, n_bwd, seed, options, adjoint=True)
    jac = np.zeros((6,) + w.shape)
    jac[1:] = j5
    if with_depth:
        p = parameters_of(cfg)
        h = depth_step if depth_step is not None else max(0.01 * p[0], 0.01)
        plus = p.copy()
        plus[0] += h
        wp, _ = _run(with_parameters(cfg, plus), n_fwd, n_bwd, seed, options, adjoint=False)
        # the simulated time span follows the depth; bins share t = 0 and their width, so
        # the shifted runs are cut or zero-padded to this run's bins
        if depth_difference == "forward":
            jac[0] = (_fit(wp, w.shape[1]) - w) / h
        else:
            minus = p.copy()
            minus[0] -= h
            wm, _ = _run(with_parameters(cfg, minus), n_fwd, n_bwd, seed, options, adjoint=False)
            jac[0] = (_fit(wp, w.shape[1]) - _fit(wm, w.shape[1])) / (2.0 * h)
    return w, jac


def _fit(w: np.ndarray, nbins: int) -> np.ndarray:
    out = np.zeros((w.shape[0], nbins))
    n = min(nbins, w.shape[1])
    out[:, :n] = w[:, :n]
    return out


def _torch():
    import torch

    return torch


class WaveformFunction:
    """``WaveformFunction.apply(params, cfg, n_fwd, n_bwd, seed, options)`` -> waveform.

    params: float64 tensor [6] (PARAMS order). The depth column is formed only when the
    depth needs a gradient."""

    _impl = None

    @classmethod
    def apply(cls, params, cfg, n_fwd, n_bwd, seed, options=None):
        if cls._impl is None:
            torch = _torch()

            class _Fn(torch.autograd.Function):
                @staticmethod
                def forward(ctx, p, cfg_, nf, nb, sd, opts):
                    vals = p.detach().cpu().double().numpy()
                    run_cfg = with_parameters(cfg_, vals)
                    w, jac = simulate_with_jacobian(
                        run_cfg, nf, nb, sd, opts, with_depth=bool(ctx.needs_input_grad[0])
                    )
                    ctx.save_for_backward(torch.from_numpy(jac))
                    return torch.from_numpy(w).to(p.device)

                @staticmethod
                def backward(ctx, g):
                    (jac,) = ctx.saved_tensors
                    grad = torch.einsum("pcb,cb->p", jac.to(g.device), g.double())
                    return grad, None, None, None, None, None

            cls._impl = _Fn
        return cls._impl.apply(params, cfg, n_fwd, n_bwd, seed, options)


def depth_difference_bias(cfg, n_fwd: int, n_bwd: int, seeds: Sequence[int], depth_step: Optional[float] = None,
                          streams: int = 4, runner=None) -> dict:
    """The forward depth difference against the central one, in expectation over seeds.

    Per seed, three plain runs with the seed's streams at depth d - h, d, d + h (h as in
    ``simulate_with_jacobian``). Per channel: the mean over seeds of the channel totals'
    forward difference and central difference, and rel_bias = mean(forward - central) /
    |mean(central)| with its paired standard error (NaN where the central difference is
    zero). runner(configs, seeds) -> waveforms replaces the device batch (tests)."""
    p0 = parameters_of(cfg)
    h = depth_step if depth_step is not None else max(0.01 * p0[0], 0.01)
    configs, run_seeds = [], []
    for s in seeds:
        for dz in (-h, 0.0, h):
            q = p0.copy()
            q[0] += dz
            configs.append(with_parameters(cfg, q))
            run_seeds.append(s)
    if runner is None:
        from pyalbsim_gb300.batch import Instance, run_batch

        inst = [Instance(c, n_fwd, n_bwd, s, None) for c, s in zip(configs, run_seeds)]
        waves, _, status, _, _ = run_batch(inst, streams=streams)
        if np.any(status != 0):
            raise RuntimeError(f"depth difference check: {int((status != 0).sum())} runs failed")
    else:
        waves = runner(configs, run_seeds)
    nb = waves[1].shape[1]
    fwd, cen = [], []
    for k in range(len(seeds)):
        wm, w0, wp = (_fit(waves[3 * k + j], nb).sum(axis=1) for j in range(3))
        fwd.append((wp - w0) / h)
        cen.append((wp - wm) / (2.0 * h))
    fwd, cen = np.array(fwd), np.array(cen)
    cm = cen.mean(axis=0)
    den = np.where(cm != 0, np.abs(cm), np.nan)
    d = fwd - cen
    se = d.std(axis=0, ddof=1) / np.sqrt(len(seeds)) if len(seeds) > 1 else np.full(4, np.nan)
    return {"forward": fwd.mean(axis=0).tolist(), "central": cm.tolist(), "step_m": h,
            "rel_bias": (d.mean(axis=0) / den).tolist(), "rel_bias_se": (se / den).tolist()}


# Relative half-steps of the central differences in ``difference_check``: a, b and g move
# paths (free-path lengths, scatter counts, directions), so their differences need steps
# that span many integrator and neighbour-set jumps; albedo and roughness leave every path
# unchanged and differ smoothly at a small step.
CHECK_STEPS = {1: 0.05, 2: 0.05, 3: 0.02, 4: 1e-3, 5: 1e-3}


def difference_check(cfg, n_fwd: int, n_bwd: int, seeds: Sequence[int], steps=None, streams: int = 4,
                     runner=None) -> dict:
    """The adjoint's columns against central differences with common random numbers, in
    expectation over seeds.

    Per seed: one adjoint run at ``cfg`` and, per parameter p in ``steps`` (PARAMS index ->
    relative half-step; default ``CHECK_STEPS``, without g on a Fournier-Forand column), two
    plain runs at p(1 +- h) with the seed's streams. Compared per parameter and channel: the
    total over bins of the column (d total / d p) and of the difference. A single seed says
    little for a, b and g (a path that moves changes its integrator step and neighbour set,
    so both estimates carry noise), hence the seeds and the paired standard error.

    runner(configs, seeds, jacobian_mask) -> (waveforms, jacobians) replaces the device
    batch (tests); by default every run goes through one ``alb_batch_run``.

    Returns {PARAMS name: {"adjoint": [4], "difference": [4], "rel_diff": [4],
    "rel_diff_se": [4]}} with rel_diff = mean(adjoint - difference) / |mean(difference)|
    and its paired standard error over seeds (NaN in channels the parameter does not
    reach)."""
    p0 = parameters_of(cfg)
    if steps is None:
        steps = dict(CHECK_STEPS)
        if getattr(cfg.water.layers[0], "henyey_greenstein_g", None) is None:
            steps.pop(3)
    if any(i == 0 for i in steps):
        raise ValueError("the depth column is itself a difference; it has no adjoint to check")
    configs, run_seeds, mask = [], [], []
    for s in seeds:
        configs.append(cfg)
        run_seeds.append(s)
        mask.append(True)
        for i, h in steps.items():
            for sign in (1.0, -1.0):
                q = p0.copy()
                q[i] *= 1.0 + sign * h
                configs.append(with_parameters(cfg, q))
                run_seeds.append(s)
                mask.append(False)
    if runner is None:
        from pyalbsim_gb300.batch import Instance, run_batch

        inst = [Instance(c, n_fwd, n_bwd, s, None) for c, s in zip(configs, run_seeds)]
        waves, jacs, status, _, _ = run_batch(inst, streams=streams, adjoint=True, jacobian_mask=mask)
        if np.any(status != 0):
            raise RuntimeError(f"difference check: {int((status != 0).sum())} runs failed")
    else:
        waves, jacs = runner(configs, run_seeds, mask)
    per = 1 + 2 * len(steps)
    S = len(seeds)
    adj = {i: np.zeros((S, 4)) for i in steps}
    dif = {i: np.zeros((S, 4)) for i in steps}
    for k in range(S):
        base = k * per
        for n, (i, h) in enumerate(steps.items()):
            adj[i][k] = jacs[base][i - 1].sum(axis=1)
            wp = waves[base + 1 + 2 * n].sum(axis=1)
            wm = waves[base + 2 + 2 * n].sum(axis=1)
            dif[i][k] = (wp - wm) / (2.0 * h * p0[i])
    out = {}
    for i in steps:
        a, d = adj[i], dif[i]
        dm = d.mean(axis=0)
        # a channel the parameter does not reach has an all-zero column and a difference of
        # summation-order rounding: no ratio
        den = np.where((dm != 0) & np.any(a != 0, axis=0), np.abs(dm), np.nan)
        diff = a - d
        se = diff.std(axis=0, ddof=1) / np.sqrt(S) if S > 1 else np.full(4, np.nan)
        out[PARAMS[i]] = {
            "adjoint": a.mean(axis=0).tolist(), "difference": dm.tolist(),
            "rel_diff": (diff.mean(axis=0) / den).tolist(), "rel_diff_se": (se / den).tolist(),
        }
    return out
