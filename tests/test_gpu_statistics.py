"""Statistical parity of the float32 tracer, the one ``run_linear``, ``run_parallel`` and the
bench run, at the configurations that are measured.

* Against the float64-geometry tracer, which reproduces the reference's runs photon by photon
  (replay fixtures, including the bench geometry), at the large single-instance geometry the
  bench runs (400 m, 20 m water, a 0.10, b 0.40, FF phase, GGX alpha 0.10, albedo 0.20,
  FOV 50 mrad, 0.05 ns bins, k = 100) and at the config-0 geometry (400 m, 5 m water, a 0.05,
  b 0.20, albedo 0.15, GGX alpha 0.05, FOV 20 mrad, 0.1 ns bins). Both tracers draw the
  same Philox blocks for the same events, so runs with the same seed share their random
  numbers: the per-seed difference of the two waveforms is a low-variance estimate of the
  float32 tracer's systematic error. Its mean over seeds, at 1 ns resolution, must be within
  1% in relative L1 of the waveform, beyond the L1 that the difference's own Monte Carlo
  noise produces (``noise``, the expected L1 of a zero-mean difference with these standard
  errors), for the summed waveform and every channel whose noise is below 0.5% (so that
  the 1% bar has power there; the surface-reflection and transmission-up channels must
  reach it).
* Against 32 runs of the reference's own ``run_linear`` at the config-0 geometry
  (``tests/golden/stats_cfg0.npz``): every populated bin in distribution
  (``fixtures.assert_statistically_equal``: 3 combined standard errors in the CLT regime, a
  Mann-Whitney rank test for every bin) and the channel totals within 3 combined standard
  errors. An L1 bar against these runs has no power: their surface-reflection totals vary by
  40% from run to run (a few backward photons landing next to the laser spot with a tiny
  k-NN radius dominate a run), so two unbiased estimates at this size already differ by
  about 36% in L1.
"""

import numpy as np
import pytest

from fixtures import assert_statistically_equal, config_from_fixture, load

pytestmark = pytest.mark.gpu

L1_BAR = 0.01
NOISE_BAR = 0.005
CHANNELS = ("bottom", "scatter", "surface_reflection", "transmission_up")


def _runs(cfg, nf, nb, seeds, precise):
    """Waveforms [runs, 4, bins] / (nf * nb), one context reset between runs (as the bench)."""
    from pyalbsim_gb300.config.gpu import GpuRunOptions
    from pyalbsim_gb300.engine import GpuEngine

    out = []
    eng = GpuEngine(cfg, GpuRunOptions(precise=precise))
    try:
        for s in seeds:
            eng.ctx.reset()
            eng.n_forward = eng.n_backward = 0
            eng.forward(nf, s)
            eng.build_maps()
            eng.backward(nb, s)
            out.append(eng.waveform_array(f64=True) / (nf * nb))
    finally:
        eng.close()
    return np.stack(out)


def _coarse(w, width):
    n = w.shape[-1] // width * width
    return w[..., :n].reshape(*w.shape[:-1], n // width, width).sum(-1)


def paired_l1(a, b, width):
    """a, b: [runs, bins] of the same seeds. Relative L1 of the mean per-seed difference
    after summing ``width`` bins, and the L1 a zero-mean difference with the same standard
    errors would show on average."""
    D, B = _coarse(a - b, width), _coarse(b, width)
    se = D.std(0, ddof=1) / np.sqrt(len(D))
    den = np.abs(B.mean(0)).sum()
    return float(np.abs(D.mean(0)).sum() / den), float(np.sqrt(2.0 / np.pi) * se.sum() / den)


def assert_paired_l1(fast, precise, width, required=("sum",)):
    """The 1% bar on the summed waveform and on every channel whose own noise resolves it
    (noise <= 0.5%); channels in ``required`` must resolve it. The others (heavy-tailed or
    small channels at this photon count) are covered by the per-bin test."""
    total = np.abs(precise.sum(1).mean(0)).sum()
    rows, failures = [], []
    series = [(CHANNELS[c], fast[:, c], precise[:, c]) for c in range(4)]
    series.append(("sum", fast.sum(1), precise.sum(1)))
    for name, a, b in series:
        share = np.abs(b.mean(0)).sum() / total
        if share == 0.0:
            continue
        l1, noise = paired_l1(a, b, width)
        rows.append(f"{name} ({share:.2%} of the waveform): L1 {l1:.3%}, noise {noise:.3%}")
        if noise > NOISE_BAR:
            if name in required:
                failures.append(f"{name}: noise {noise:.3%} above {NOISE_BAR:.1%}")
            continue
        if l1 > L1_BAR + noise:
            failures.append(f"{name}: L1 {l1:.3%} above {L1_BAR:.0%} + noise {noise:.3%}")
    assert not failures, (failures, rows)
    return rows


def _fast_vs_precise(cfg, nf, nb, seeds, width, required):
    fast = _runs(cfg, nf, nb, seeds, precise=False)
    precise = _runs(cfg, nf, nb, seeds, precise=True)
    st = {"per_run": precise, "mean": precise.mean(0), "se": precise.std(0, ddof=1) / np.sqrt(len(precise))}
    assert_statistically_equal(fast, st)  # conservative for paired runs
    return assert_paired_l1(fast, precise, width, required)


def test_fast_tracer_matches_precise_at_the_bench_geometry(gpu_available):
    """The large single-instance scene, 1e6 + 2.5e5 photons, 32 seeds; 1 ns = 20 bins. The
    surface-reflection and transmission-up channels and the sum must resolve the 1% bar."""
    from pyalbsim_gb300.workloads import large

    rows = _fast_vs_precise(large(), 1_000_000, 250_000, range(500, 532), width=20,
                            required=("surface_reflection", "transmission_up", "sum"))
    print("bench geometry, fast vs precise:", "; ".join(rows))


def test_fast_tracer_matches_precise_at_config0(gpu_available):
    """The config-0 geometry, 1e6 + 2.5e5 photons, 32 seeds; 1 ns = 10 bins."""
    cfg = config_from_fixture(load("stats_cfg0.npz"))
    rows = _fast_vs_precise(cfg, 1_000_000, 250_000, range(700, 732), width=10,
                            required=("surface_reflection", "transmission_up", "sum"))
    print("config 0, fast vs precise:", "; ".join(rows))


@pytest.mark.parametrize("precise", [False, True], ids=["fast", "precise"])
def test_a_photon_leaves_the_water_once(gpu_available, precise):
    """A forward photon that leaves the water through the surface is in the air for good, so
    it makes at most one transmission-up record (at 400 m a float32 height is quantised as
    coarsely as a grazing photon's vertical step; a transmitted photon left on the surface
    plane would exit again)."""
    from pyalbsim_gb300.config.gpu import GpuRunOptions
    from pyalbsim_gb300.engine import GpuEngine
    from pyalbsim_gb300.workloads import large

    eng = GpuEngine(large(), GpuRunOptions(precise=precise))
    try:
        eng.keep_record_ids(True)
        eng.forward(200_000, 501)
        ids = eng.ctx.export_map(3)[6]
    finally:
        eng.close()
    assert len(ids) > 100_000
    assert np.bincount(ids).max() == 1


def test_fast_tracer_matches_reference_runs_at_config0(gpu_available):
    """32 Philox runs of the float32 tracer against the 32 runs of the reference's
    run_linear at the config-0 geometry, the same photon counts per run (8000 + 2000).

    The run counts are equal on purpose. The late bins of the bottom, scatter and
    transmission-up channels are right-skewed across runs (rare long paths carry large
    contributions), so the mean and standard error of the smaller sample run low more often
    than not: with 128 runs on one side and 32 on the other, even two samples of the same
    algorithm (the oracle against the float32 tracer) show 20-40 bins beyond 3 standard
    errors, all in favour of the larger sample, while 32 against 32 shows none beyond the
    test's allowance."""
    st = load("stats_cfg0.npz")
    cfg = config_from_fixture(st)
    runs, nf, nb = int(st["runs"]), int(st["n_fwd"]), int(st["n_bwd"])
    lo, width = int(st["bin0"]), st["per_run"].shape[-1]
    w = _runs(cfg, nf, nb, range(9000, 9000 + runs), precise=False)
    assert w.shape[-1] == int(st["nbins"])
    outside = np.delete(w, np.s_[lo:lo + width], axis=-1)
    # nothing lands outside the window the reference runs populate, beyond a sliver of the
    # total (a rare long path the 32 reference runs did not sample)
    assert np.abs(outside).sum() <= 1e-3 * np.abs(w).sum()
    mine = w[..., lo:lo + width]
    ref = st["per_run"].astype(np.float64)
    assert_statistically_equal(mine, {"per_run": ref, "mean": st["mean"], "se": st["se"]})
    a, b = mine.sum(-1), ref.sum(-1)  # channel totals per run
    se = np.sqrt(a.var(0, ddof=1) / len(a) + b.var(0, ddof=1) / len(b))
    z = np.abs(a.mean(0) - b.mean(0)) / np.where(se > 0, se, 1.0)
    assert np.all(z < 3.0), (a.mean(0), b.mean(0), se)
    print("config 0 vs reference, channel totals (GPU, reference, z):",
          [(float(x), float(y), float(t)) for x, y, t in zip(a.mean(0), b.mean(0), z)])
