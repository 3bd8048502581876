"""Waveform inversion (extension: the reference has no gradients).

Each target waveform is fitted by Adam over the six parameters (depth, a, b, HG g,
seafloor albedo, roughness) from a common initial guess. Every iteration runs all targets
in one ``alb_batch_run``. Per target there is an adjoint instance at its current
parameters, which gives the waveform and five Jacobian columns, and a plain instance at
depth + h, which gives the depth column by a common-random-number forward difference
(``depth_difference="central"``: two plain instances at depth +- h). All share the
iteration's Philox key, which changes from iteration to iteration (a stochastic gradient).

The loss compares the scaled simulated waveform s w with the target counts c, where c is
the target waveform scaled to ``peak`` counts with Poisson shot noise and s is the same
scale:
- ``loss="mse"`` is ``sum (s w - c)^2``. The surface return dominates it.
- ``loss="log"`` is ``sum (ln(1 + s w) - ln(1 + c))^2``. It weighs the weak seafloor return
  comparably.

Adam works on u = ln(theta / theta_0), so every parameter moves by relative steps. g stays
below 0.99. With ``resample=False`` every iteration reuses one Philox key: a fixed
common-random-number objective.

The loss has no depth slope while the simulated seafloor return does not overlap the
target's, so ``depth_grid`` (depths in m) starts every target at the grid depth of lowest
loss, the other parameters at the initial guess. Those runs form one more batch.
``depth_init="bottom_peak"`` starts it from the target itself instead, the way a
bathymetric lidar reads a depth: the time of the seafloor return's peak in the target's
seafloor channel, converted to a depth by the peak shift of two model runs at the initial
guess and 5 m deeper (the seafloor return moves about 2 n / c seconds per metre; the
calibration carries the scene's bin width, refractive index and view angles). A target
whose seafloor return holds too few counts to locate keeps its start and is reported as
undetectable.
"""

from __future__ import annotations

import dataclasses
import math
from typing import Dict, Optional, Sequence

import numpy as np

from pyalbsim_gb300.adjoint import with_parameters
from pyalbsim_gb300.batch import Instance, RANGES, run_batch, surface_gate
from pyalbsim_gb300.workloads import small

INITIAL = np.array([10.0, 0.1, 0.3, 0.9, 0.2, math.sqrt(0.1)])
# counts added to the scaled waveform in the Poisson likelihood: bins the model leaves empty
# while the target holds counts keep a finite loss
POISSON_FLOOR = 1e-2


def gated_base(length: float = 400e-9):
    """The small scene with an HG layer and a window long enough for a 40 m seafloor."""
    base = small(hg=0.9)
    return dataclasses.replace(base, waveform_gate=surface_gate(base, length=length))


def hypercube_targets(n: int, seed: int = 4) -> np.ndarray:
    """n six-parameter points at LatinHypercube(d=7, seed) over the sweep ranges (the
    field-of-view column is drawn and not used: the fit keeps the base receiver)."""
    from scipy.stats import qmc

    u = qmc.LatinHypercube(d=7, seed=seed).random(n)
    lo = np.array([r[0] for r in RANGES.values()])
    hi = np.array([r[1] for r in RANGES.values()])
    p = lo + u * (hi - lo)
    p[:, 5] = np.sqrt(p[:, 5])  # GGX alpha -> roughness
    return p[:, :6]


def _clip(theta: np.ndarray) -> np.ndarray:
    t = theta.copy()
    t[..., 3] = np.minimum(t[..., 3], 0.99)
    t[..., 0] = np.maximum(t[..., 0], 0.2)
    t[..., 4] = np.minimum(t[..., 4], 1.0)
    return t


def fit(
    targets: np.ndarray,
    iters: int = 200,
    lr: float = 1e-2,
    photons: int = 1_000_000,
    peak: float = 1e4,
    seed: int = 4,
    streams: int = 8,
    base=None,
    initial: Optional[Sequence[float]] = None,
    depth_step: float = 0.05,
    loss: str = "log",
    resample: bool = False,
    depth_grid: Optional[Sequence[float]] = None,
    fixed: Optional[Sequence[bool]] = None,
    prior_sigma: Optional[Sequence[Optional[float]]] = None,
    depth_difference: str = "forward",
    depth_init: Optional[str] = None,
) -> Dict:
    """Fit every row of ``targets`` (n x 6). Returns final parameters, depth errors and the
    per-iteration mean data loss.

    depth_difference: "forward" (one plain instance at depth + depth_step per target) or
    "central" (two, at depth +- depth_step) for the depth column of the gradient.

    depth_init: None, or "bottom_peak" to start each target's depth from the peak of its
    seafloor channel (module docstring); the result then holds ``depth_detectable``.

    loss: "log" (squared difference of log(1 + counts)), "mse", or "poisson" (the negative
    log-likelihood of the Poisson counts, sum(lambda - counts ln lambda), lambda the scaled
    waveform plus a floor of ``POISSON_FLOOR`` counts).

    From one waveform the depth trades against attenuation and scattering, so the free
    six-parameter fit is not identifiable. Two ways to constrain it:
    ``fixed``: six booleans; a fixed parameter stays at its initial value.
    ``prior_sigma``: six standard deviations (None = flat) of Gaussian priors on
    u = ln(theta / initial); the fit then minimises the data loss plus sum((u / sigma)^2) / 2.
    With the Poisson loss that is the maximum a posteriori estimate; with the others the
    sigmas are relative to the loss's own scale."""
    base = base or gated_base()
    targets = np.asarray(targets, dtype=np.float64)
    n = len(targets)
    nb = max(photons // 4, 1)
    rng = np.random.default_rng(seed)
    # targets: one noiseless run each (own keys), scaled to the peak, Poisson shot noise
    tinst = [Instance(with_parameters(base, targets[i]), photons, nb, (seed << 40) + i, targets[i]) for i in range(n)]
    tw, _, st, _, _ = run_batch(tinst, streams=streams)
    if np.any(st != 0):
        raise RuntimeError(f"target simulation failed: {st}")
    scale = np.array([peak / max(float(w.max()), 1e-300) for w in tw])
    counts = [rng.poisson(np.clip(scale[i] * tw[i], 0, None)).astype(np.float64) for i in range(n)]

    theta0 = np.array(initial if initial is not None else INITIAL, dtype=np.float64)
    u = np.zeros((n, 6))
    if depth_difference not in ("forward", "central"):
        raise ValueError("depth_difference must be 'forward' or 'central'")
    free = np.ones(6) if fixed is None else 1.0 - np.asarray(fixed, dtype=np.float64)
    if free.shape != (6,):
        raise ValueError("fixed needs six entries")
    inv_var = np.zeros(6)
    if prior_sigma is not None:
        if len(prior_sigma) != 6:
            raise ValueError("prior_sigma needs six entries")
        for k, sd in enumerate(prior_sigma):
            if sd is not None:
                if not sd > 0:
                    raise ValueError("prior standard deviations must be positive")
                inv_var[k] = 1.0 / (sd * sd)

    if loss not in ("log", "mse", "poisson"):
        raise ValueError(f"unknown loss {loss!r}")

    def loss_of(wi, i):
        return loss_and_grad(wi, i)[0]

    def loss_and_grad(wi, i):
        """(loss, d loss / d waveform) of one target."""
        sw = np.clip(scale[i] * wi, 0.0, None)
        if loss == "mse":
            r = sw - counts[i]
            return float((r ** 2).sum()), 2.0 * scale[i] * r
        if loss == "poisson":
            lam = sw + POISSON_FLOOR
            c = counts[i]
            return float((lam - c * np.log(lam)).sum()), scale[i] * (1.0 - c / lam)
        r = np.log1p(sw) - np.log1p(counts[i])
        return float((r ** 2).sum()), 2.0 * r * scale[i] / (1.0 + sw)

    detectable = np.ones(n, dtype=bool)
    if depth_init is not None:
        if depth_init != "bottom_peak":
            raise ValueError(f"unknown depth_init {depth_init!r}")
        if free[0]:
            detectable = _bottom_peak_start(base, theta0, counts, photons, nb, seed, streams, u)
    if depth_grid is not None:
        grid = np.asarray(depth_grid, dtype=np.float64)
        key = (seed << 40) + (1 << 32)
        ginst = []
        for i in range(n):
            for dz in grid:
                q = theta0.copy()
                q[0] = dz
                ginst.append(Instance(with_parameters(base, q), photons, nb, key, q))
        gw, _, gst, _, _ = run_batch(ginst, streams=streams)
        for i in range(n):
            ls = [loss_of(gw[i * len(grid) + j], i) if gst[i * len(grid) + j] == 0 else np.inf
                  for j in range(len(grid))]
            # a depth read from the target's own seafloor return takes precedence
            if free[0] and not (depth_init is not None and detectable[i]):
                u[i, 0] = math.log(grid[int(np.argmin(ls))] / theta0[0])
    m_ = np.zeros((n, 6))
    v_ = np.zeros((n, 6))
    b1, b2, eps = 0.9, 0.999, 1e-8
    history = []
    for it in range(iters):
        theta = _clip(theta0 * np.exp(u))
        key = (seed << 40) + (1 << 32) + (it if resample else 0)
        shifts = ((1.0,) if depth_difference == "forward" else (1.0, -1.0)) if free[0] else ()
        per = 1 + len(shifts)  # the depth runs only while the depth is free
        inst = []
        for i in range(n):
            inst.append(Instance(with_parameters(base, theta[i]), photons, nb, key, theta[i]))
            for sgn in shifts:
                q = theta[i].copy()
                q[0] += sgn * depth_step
                inst.append(Instance(with_parameters(base, q), photons, nb, key, q))
        w, jac, st, _, _ = run_batch(inst, streams=streams, adjoint=True,
                                     jacobian_mask=[k % per == 0 for k in range(len(inst))])
        grads = np.zeros((n, 6))
        losses = np.zeros(n)
        for i in range(n):
            k = per * i
            if np.any(st[k:k + per] != 0):
                raise RuntimeError(f"iteration {it}, target {i}: status {st[k:k + per]}")
            losses[i], dl_dw = loss_and_grad(w[k], i)
            grads[i, 1:] = np.einsum("pcb,cb->p", jac[k], dl_dw)
            if free[0]:
                lp = loss_and_grad(w[k + 1], i)[0]
                if depth_difference == "forward":
                    grads[i, 0] = (lp - losses[i]) / depth_step
                else:
                    lm = loss_and_grad(w[k + 2], i)[0]
                    grads[i, 0] = (lp - lm) / (2.0 * depth_step)
        gu = (grads * theta + u * inv_var) * free  # d (L + prior) / d u for theta = theta0 e^u
        m_ = b1 * m_ + (1 - b1) * gu
        v_ = b2 * v_ + (1 - b2) * gu * gu
        mh = m_ / (1 - b1 ** (it + 1))
        vh = v_ / (1 - b2 ** (it + 1))
        u -= lr * mh / (np.sqrt(vh) + eps)
        history.append(float(losses.mean()))
    final = _clip(theta0 * np.exp(u))
    out = {
        "params": final,
        "targets": targets,
        "depth_error": final[:, 0] - targets[:, 0],
        "loss_history": np.array(history),
    }
    if depth_init is not None:
        out["depth_detectable"] = detectable
    return out


# counts at the smoothed seafloor peak below which a target's seafloor return is not located
BOTTOM_PEAK_MIN_COUNTS = 5.0
CALIBRATION_STEP = 5.0  # m between the two model runs that convert a peak shift to a depth


def _smoothed_peak(w: np.ndarray, width: int = 5) -> tuple:
    """(bin, height) of the maximum of w after a centred box filter of ``width`` bins."""
    k = np.ones(width) / width
    sm = np.convolve(w, k, mode="same")
    b = int(np.argmax(sm))
    return b, float(sm[b])


def _bottom_peak_start(base, theta0, counts, photons, nb, seed, streams, u) -> np.ndarray:
    """Sets u[i, 0] from the seafloor-channel peak of each target's counts (channel 0);
    returns which targets had a locatable seafloor return. One batch: the model at the
    initial guess and 5 m deeper, on one Philox key."""
    n = len(counts)
    d0 = float(theta0[0])
    key = (seed << 40) + (3 << 32)
    q0 = theta0.copy()
    q1 = theta0.copy()
    q1[0] = d0 + CALIBRATION_STEP
    cw, _, cst, _, _ = run_batch([Instance(with_parameters(base, q0), photons, nb, key, q0),
                                  Instance(with_parameters(base, q1), photons, nb, key, q1)], streams=streams)
    if np.any(cst != 0):
        raise RuntimeError(f"depth calibration runs failed: {cst}")
    b0, _ = _smoothed_peak(np.asarray(cw[0])[0])
    b1, _ = _smoothed_peak(np.asarray(cw[1])[0])
    bins_per_m = (b1 - b0) / CALIBRATION_STEP
    ok = np.zeros(n, dtype=bool)
    if not bins_per_m > 0:
        return ok
    for i in range(n):
        bt, h = _smoothed_peak(np.asarray(counts[i])[0])
        if h < BOTTOM_PEAK_MIN_COUNTS:
            continue
        depth = max(d0 + (bt - b0) / bins_per_m, 0.2)
        u[i, 0] = math.log(depth / d0)
        ok[i] = True
    return ok
