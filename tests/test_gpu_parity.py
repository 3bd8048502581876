"""GPU parity tests: the CUDA path through the C ABI against the reference's recorded runs
(replay mode), the oracle (same Philox streams), scipy's KDTree answers and independent
reference runs (statistics). All tests here need a GB300 and libalbgpu.so."""

import numpy as np
import pytest

from fixtures import assert_statistically_equal, config_from_fixture, load, replay_streams
from oracle.oracle import oracle_run
from pyalbsim_gb300.engine import GpuEngine
from pyalbsim_gb300.scene import build_scene

pytestmark = pytest.mark.gpu

REPLAYS = ["small", "twolayer", "cfg0", "profiled"]
# Tolerances: FP32 arithmetic on the device vs float64 in the reference.
REL_WAVEFORM_L1 = 1e-5


def _engine(cfg, ids=True, exits=True, precise=True):
    from pyalbsim_gb300.config.gpu import GpuRunOptions

    eng = GpuEngine(cfg, GpuRunOptions(precise=precise))
    if ids:
        eng.keep_record_ids(True)
    if exits:
        eng.keep_exit_states(True)
    return eng


@pytest.fixture(scope="module", params=REPLAYS)
def gpu_replay(request, gpu_available):
    d = load(f"replay_{request.param}.npz")
    cfg = config_from_fixture(d)
    nf, nb = int(d["n_fwd"]), int(d["n_bwd"])
    eng = _engine(cfg)
    eng.forward(nf, 0, replay=replay_streams(d, "fwd"))
    fexit = eng.ctx.exit_states(nf)
    maps = {c: eng.ctx.export_map(c) for c in range(4)}  # unsorted (record) order
    eng.build_maps()
    eng.backward(nb, 0, replay=replay_streams(d, "bwd"))
    bexit = eng.ctx.exit_states(nb)
    queries = {k: eng.ctx.export_queries(k) for k in range(3)}
    wf = eng.waveform_array(f64=True)
    heat = eng.heatmaps()
    orc = oracle_run(eng.scene, nf, nb, replay_fwd=replay_streams(d, "fwd"), replay_bwd=replay_streams(d, "bwd"))
    out = dict(d=d, maps=maps, fexit=fexit, bexit=bexit, queries=queries, wf=wf, heat=heat, orc=orc, eng=eng)
    yield request.param, out
    eng.close()


def test_replay_maps_match_reference(gpu_replay):
    name, o = gpu_replay
    d = o["d"]
    for c in range(4):
        pos, dr, e, t, fwi, sfi, pid = o["maps"][c]
        if f"map{c}_pos" not in d:
            assert len(e) == 0
            continue
        assert len(e) == len(d[f"map{c}_energy"]), (name, c)
        ia = np.lexsort((t, pid))
        ib = np.lexsort((d[f"map{c}_time"], d[f"map{c}_ids"]))
        np.testing.assert_array_equal(pid[ia], d[f"map{c}_ids"][ib])
        np.testing.assert_array_equal(t[ia], d[f"map{c}_time"][ib])
        np.testing.assert_allclose(e[ia], d[f"map{c}_energy"][ib], rtol=1e-6)
        np.testing.assert_allclose(pos[ia], d[f"map{c}_pos"][ib], rtol=1e-5, atol=1e-5)
        np.testing.assert_allclose(dr[ia], d[f"map{c}_dir"][ib], rtol=0, atol=1e-5)


def test_replay_exit_states_match_reference(gpu_replay):
    name, o = gpu_replay
    d = o["d"]
    for p, ex in (("fwd", o["fexit"]), ("bwd", o["bexit"])):
        np.testing.assert_allclose(ex["energy"], d[f"{p}_final_energy"], rtol=1e-6)
        np.testing.assert_array_equal(ex["time"], d[f"{p}_final_time"])
        np.testing.assert_array_equal(ex["tau_target"], d[f"{p}_final_tau_target"])
        np.testing.assert_allclose(ex["tau"], d[f"{p}_final_tau"], rtol=1e-5, atol=1e-5)
        np.testing.assert_allclose(ex["pos"], d[f"{p}_final_pos"], rtol=1e-5, atol=1e-4)
        np.testing.assert_allclose(ex["dir"], d[f"{p}_final_dir"], rtol=0, atol=1e-5)


def test_replay_queries_match_reference(gpu_replay):
    name, o = gpu_replay
    q = o["d"]["queries"]
    for kind in range(3):
        mine = o["queries"][kind]
        ref = q[q[:, 0] == kind]
        assert len(mine["energy"]) == len(ref), (name, kind)
        if len(ref) == 0:
            continue
        ia = np.lexsort((mine["time"], mine["id"]))
        ib = np.lexsort((ref[:, 9], ref[:, 1]))
        np.testing.assert_array_equal(mine["id"][ia], ref[ib, 1].astype(np.int64))
        np.testing.assert_array_equal(mine["time"][ia], ref[ib, 9].astype(np.float32))
        np.testing.assert_allclose(mine["pos"][ia], ref[ib, 2:5], rtol=1e-6, atol=1e-5)


def test_replay_waveform_matches_reference(gpu_replay):
    """Waveform vs the reference's float64-accumulated waveform: L1 <= 1e-5 per channel."""
    name, o = gpu_replay
    ref = o["d"]["waveform64"]
    for c in range(4):
        den = np.abs(ref[c]).sum()
        if den == 0:
            continue
        l1 = np.abs(o["wf"][c] - ref[c]).sum() / den
        assert l1 < REL_WAVEFORM_L1, (name, c, l1)


def test_replay_waveform_matches_oracle(gpu_replay):
    name, o = gpu_replay
    orc = o["orc"]["waveform"]
    for c in range(4):
        den = np.abs(orc[c]).sum()
        if den:
            assert np.abs(o["wf"][c] - orc[c]).sum() / den < REL_WAVEFORM_L1, (name, c)


def test_replay_rk_matches_oracle(gpu_replay):
    """k-th neighbour distance of every gather equals the oracle's (brute-force) one."""
    name, o = gpu_replay
    orc = o["orc"]
    for ch, kind in ((0, 0), (1, 1), (2, 2), (3, 2)):
        if ch not in orc["rk"]:
            continue
        mine = o["queries"][kind]
        ref_q = orc["queries"][kind]
        key_m = np.lexsort((mine["time"], mine["id"]))
        key_r = np.lexsort((ref_q["time"], ref_q["photon"]))
        rk_m = (mine["rk2"] if ch == 3 else mine["rk"])[key_m]
        np.testing.assert_allclose(rk_m, orc["rk"][ch][key_r], rtol=1e-6, atol=1e-9)


def test_replay_heatmaps(gpu_replay):
    name, o = gpu_replay
    d = o["d"]
    if o["heat"] is None or "heat_radius" not in d:
        return
    np.testing.assert_array_equal(o["heat"].scatter_radius_heatmap, d["heat_radius"])
    for mine, key in ((o["heat"].water_heatmap, "heat_water"), (o["heat"].seafloor_heatmap, "heat_floor")):
        ref = d[key].astype(np.float64)
        assert np.abs(mine - ref).sum() / np.abs(ref).sum() < 1e-4, key


def test_knn_neighbour_sets_bit_exact(gpu_available):
    kn = load("knn.npz")
    eng = GpuEngine(config_from_fixture(load("replay_small.npz")))
    try:
        for name in ("planar", "cloud", "cloud_k16"):
            pts, qs, k = kn[f"{name}_points"], kn[f"{name}_queries"], int(kn[f"{name}_k"])
            dist, idx = eng.ctx.knn(pts, qs, k)
            np.testing.assert_allclose(dist, kn[f"{name}_dist"], rtol=1e-12, atol=0)
            ref_idx, ref_d = kn[f"{name}_idx"], kn[f"{name}_dist"]
            for i in range(len(qs)):
                strict = set(ref_idx[i][ref_d[i] < ref_d[i][-1]])  # exclude exact ties at r_k
                assert strict <= set(idx[i]), (name, i)
    finally:
        eng.close()


@pytest.mark.parametrize("leaves,kinds_expected", [(2048 + 512 + 5, {128, 64}), (2048 + 256 + 5, {128, 32}),
                                                   (2048 + 100, {128, 8})])
def test_knn_every_cell_kind_matches_kdtree(gpu_available, leaves, kinds_expected):
    """Map sizes whose left-balanced k-d tree ends in perfect cells of 128 leaves and of 64
    (2048 + 512 + 5 leaves) or 32 (2048 + 256 + 5), or in multi-leaf general cells
    (2048 + 100), plus single leaves and a partial last leaf, so every kind of per-CTA cell
    kernel orders records. A third of the points sit on
    a coarse lattice and a tenth are exact duplicates, so many records share a node's 16-bit
    coordinate at its cut (the ties the partition ranks by position). Neighbour sets match
    scipy's cKDTree except for exact ties at the k-th distance."""
    sp = pytest.importorskip("scipy.spatial")

    def cells(c, depth, D):  # leaf counts of the per-CTA cells: nodes at depth D, or single leaves
        if depth == D or c <= 1:
            return [c]
        left = 1 << ((c - 1).bit_length() - 1)
        return cells(left, depth + 1, D) + cells(c - left, depth + 1, D)

    kinds = set(cells(leaves, 0, (leaves - 1).bit_length() - 7))
    assert kinds_expected <= kinds and kinds - {32, 64, 128}, kinds
    rng = np.random.default_rng(leaves)
    m = 32 * leaves - 11
    pts = rng.normal(scale=[0.5, 3.0, 0.5], size=(m, 3)) + [0.0, -405.0, 0.0]
    lat = rng.random(m) < 0.33
    pts[lat] = np.round(pts[lat] * 10.0) / 10.0
    dup = rng.random(m) < 0.1
    pts[dup] = pts[rng.integers(0, m, int(dup.sum()))]
    pts = pts.astype(np.float32)
    near = pts[rng.integers(0, m, 800)].astype(np.float64) + rng.normal(scale=0.03, size=(800, 3))
    far = np.stack([rng.uniform(-20, 20, 200), rng.uniform(-420, -390, 200), rng.uniform(-20, 20, 200)], 1)
    qs = np.concatenate([near, far])
    eng = GpuEngine(config_from_fixture(load("replay_small.npz")))
    try:
        for k in (100, 7):
            dist, idx = eng.ctx.knn(pts, qs, k)
            ref_d, ref_i = sp.cKDTree(pts.astype(np.float64)).query(qs, k)
            np.testing.assert_allclose(dist, ref_d, rtol=1e-12, atol=0)
            for i in range(len(qs)):
                strict = set(ref_i[i][ref_d[i] < ref_d[i][-1]])
                assert strict <= set(idx[i]), (leaves, k, i)
    finally:
        eng.close()


@pytest.mark.parametrize("shape", ["cloud", "planar"])
def test_knn_large_map_matches_kdtree(gpu_available, shape):
    """Maps large enough for the streaming partition levels of the index build (3e6 points:
    more than ten levels above the per-CTA cells): every query's k nearest match scipy's
    cKDTree (float64 distances on the float32 points; sets agree except for exact ties at
    the k-th distance). Includes far queries, whose neighbours crowd at nearly one distance."""
    sp = pytest.importorskip("scipy.spatial")
    rng = np.random.default_rng(11)
    m, k = 3_000_000, 100
    if shape == "cloud":
        pts = rng.normal(scale=[0.4, 5.0, 0.4], size=(m, 3)) + [0.0, -410.0, 0.0]
    else:
        r = 0.4 * np.sqrt(rng.random(m))
        a = 2 * np.pi * rng.random(m)
        pts = np.stack([r * np.cos(a), np.full(m, -400.0), r * np.sin(a)], 1)
    pts = pts.astype(np.float32)
    near = pts[rng.integers(0, m, 1500)].astype(np.float64) + rng.normal(scale=0.05, size=(1500, 3))
    far = np.stack([rng.uniform(-40, 40, 500), np.full(500, -400.0), rng.uniform(-40, 40, 500)], 1)
    if shape == "cloud":
        far[:, 1] = rng.uniform(-430, -390, 500)
    qs = np.concatenate([near, far])
    eng = GpuEngine(config_from_fixture(load("replay_small.npz")))
    try:
        dist, idx = eng.ctx.knn(pts, qs, k)
    finally:
        eng.close()
    ref_d, ref_i = sp.cKDTree(pts.astype(np.float64)).query(qs, k)
    np.testing.assert_allclose(dist, ref_d, rtol=1e-12, atol=0)
    for i in range(len(qs)):
        strict = set(ref_i[i][ref_d[i] < ref_d[i][-1]])
        assert strict <= set(idx[i]), (shape, i)


def _philox_run(cfg, nf, nb, seed, ids=True, precise=True):
    eng = _engine(cfg, ids=ids, exits=True, precise=precise)
    eng.forward(nf, seed)
    fexit = eng.ctx.exit_states(nf)
    maps = {c: eng.ctx.export_map(c) for c in range(4)}
    eng.build_maps()
    eng.backward(nb, seed)
    wf = eng.waveform_array(f64=True)
    eng.close()
    return fexit, maps, wf


def test_philox_matches_oracle_photon_by_photon(gpu_available):
    """Same Philox streams on both sides: identical records, exit states and waveform."""
    d = load("replay_small.npz")
    cfg = config_from_fixture(d)
    nf, nb, seed = 4000, 1000, 1234567
    fexit, maps, wf = _philox_run(cfg, nf, nb, seed)
    scene = build_scene(cfg)
    orc = oracle_run(scene, nf, nb, seed=seed)
    np.testing.assert_array_equal(fexit["time"], orc["fwd_exit"]["time"])
    np.testing.assert_allclose(fexit["pos"], orc["fwd_exit"]["pos"], rtol=1e-5, atol=1e-4)
    for c in range(4):
        pos, dr, e, t, fwi, sfi, pid = maps[c]
        om = orc["maps"][c]
        assert len(e) == len(om["energy"]), c
        ia = np.lexsort((t, pid))
        ib = np.lexsort((om["time"], om["photon"]))
        np.testing.assert_array_equal(pid[ia], om["photon"][ib])
        np.testing.assert_array_equal(t[ia], om["time"][ib])
        np.testing.assert_allclose(pos[ia], om["pos"][ib], rtol=1e-5, atol=1e-5)
    for c in range(4):
        den = np.abs(orc["waveform"][c]).sum()
        if den:
            assert np.abs(wf[c] - orc["waveform"][c]).sum() / den < REL_WAVEFORM_L1, c


@pytest.mark.parametrize("precise", [True, False], ids=["precise", "fast"])
def test_waveform_bit_identical_run_to_run(gpu_available, precise):
    """Order-independent fixed-point accumulation: two runs give the same bits."""
    cfg = config_from_fixture(load("replay_small.npz"))
    a = _philox_run(cfg, 20000, 5000, 99, ids=False, precise=precise)[2]
    b = _philox_run(cfg, 20000, 5000, 99, ids=False, precise=precise)[2]
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("precise", [True, False], ids=["precise", "fast"])
def test_philox_statistics_match_reference(gpu_available, precise):
    """32 Philox runs against 32 independent reference runs (N_f*N_b-normalised): bins in
    the CLT regime within 3 combined standard errors, every bin's per-run distribution
    equal under a Mann-Whitney test (fixtures.assert_statistically_equal)."""
    st = load("stats_small.npz")
    cfg = config_from_fixture(st)
    runs, nf, nb = 32, int(st["n_fwd"]), int(st["n_bwd"])
    waves = np.stack(
        [_philox_run(cfg, nf, nb, 5000 + r, ids=False, precise=precise)[2] / (nf * nb) for r in range(runs)]
    )
    assert_statistically_equal(waves, st)


def test_fast_and_precise_agree_in_distribution(gpu_available):
    """The float32 tracer against the float64-geometry tracer at 40x the reference's
    photon count: channel totals within 4 combined standard errors over 8 seeds each."""
    cfg = config_from_fixture(load("stats_small.npz"))
    nf, nb = 120000, 30000
    tot = {}
    for precise in (True, False):
        tot[precise] = np.stack(
            [_philox_run(cfg, nf, nb, 300 + r, ids=False, precise=precise)[2].sum(1) / (nf * nb) for r in range(8)]
        )
    a, b = tot[True], tot[False]
    se = np.sqrt(a.var(0, ddof=1) / 8 + b.var(0, ddof=1) / 8)
    assert np.all(np.abs(a.mean(0) - b.mean(0)) < 4 * se + 1e-30), (a.mean(0), b.mean(0), se)


def test_fast_and_precise_agree_in_distribution_profiled(gpu_available):
    """Depth-profiled layers: the float32 tracer (one step at a time in profiled layers)
    against the float64-geometry tracer, channel totals within 4 combined standard errors
    over 8 seeds each."""
    cfg = config_from_fixture(load("replay_profiled.npz"))
    nf, nb = 40000, 10000
    tot = {}
    for precise in (True, False):
        tot[precise] = np.stack(
            [_philox_run(cfg, nf, nb, 700 + r, ids=False, precise=precise)[2].sum(1) / (nf * nb) for r in range(8)]
        )
    a, b = tot[True], tot[False]
    se = np.sqrt(a.var(0, ddof=1) / 8 + b.var(0, ddof=1) / 8)
    assert np.all(np.abs(a.mean(0) - b.mean(0)) < 4 * se + 1e-30), (a.mean(0), b.mean(0), se)


def test_philox_profiled_matches_oracle(gpu_available):
    """Same Philox streams, profiled layers: the precise tracer and the oracle agree on the
    waveform within the parity tolerance."""
    cfg = config_from_fixture(load("replay_profiled.npz"))
    nf, nb = 3000, 800
    wf = _philox_run(cfg, nf, nb, 41, ids=False, precise=True)[2]
    orc = oracle_run(build_scene(cfg), nf, nb, seed=41)
    for c in range(4):
        den = np.abs(orc["waveform"][c]).sum()
        if den:
            assert np.abs(wf[c] - orc["waveform"][c]).sum() / den < REL_WAVEFORM_L1, c


def test_forward_after_build_restores_the_store(gpu_available):
    """A forward trace after the maps were built brings the records back from the index into
    the append store (interleaved halves) before it appends: the waveform equals that of
    the same photons traced before a single build, bit for bit."""
    cfg = config_from_fixture(load("replay_small.npz"))
    a, b = GpuEngine(cfg), GpuEngine(cfg)
    try:
        a.forward(3000, 5)
        a.build_maps()
        a.forward(2000, 5)  # photons 3000..4999 after the index build
        a.backward(800, 6)
        b.forward(3000, 5)
        b.forward(2000, 5)
        b.backward(800, 6)
        wa, wb = a.waveform_array(f64=True), b.waveform_array(f64=True)
        assert np.abs(wb).sum() > 0
        assert np.array_equal(wa, wb)
    finally:
        a.close()
        b.close()


def test_too_few_photons_raises_index_error(gpu_available):
    """Reference quirk: a gather on a map with fewer than k records raises IndexError."""
    cfg = config_from_fixture(load("replay_small.npz"))
    eng = GpuEngine(cfg)
    try:
        eng.forward(10, 1)  # fewer surface records than k=32
        eng.build_maps()
        with pytest.raises(IndexError):
            eng.backward(100, 1)
    finally:
        eng.close()


def test_drop_in_run_linear_and_run_parallel(gpu_available):
    from pyalbsim_gb300.config import RunConfig
    from pyalbsim_gb300.execution.linear import run_linear
    from pyalbsim_gb300.execution.parallel import run_parallel
    from pyalbsim_gb300.photon_mapping.photon_type import PhotonType

    cfg = config_from_fixture(load("replay_small.npz"))
    rc = RunConfig(photons_per_batch_forward=2000, photons_per_batch_backward=500, batches_forward=2, batches_backward=2)
    w = run_linear(cfg, rc, rng=np.random.default_rng(0))
    assert set(w) == set(PhotonType)
    steps = build_scene(cfg).steps
    for arr in w.values():
        assert arr.dtype == np.float32 and arr.shape == (2 * steps,)
        assert np.all(arr >= 0)
    w2 = run_linear(cfg, rc, rng=np.random.default_rng(0))
    for t in w:
        np.testing.assert_array_equal(w[t], w2[t])
    wave, maps, heat = run_parallel(cfg, rc, seed=5)
    assert set(wave) == set(PhotonType)
    # fixed seed: every forward batch is the same photons (reference behaviour)
    sr = maps[PhotonType.SURFACE_REFLECTION]
    n = len(sr.energies)
    assert n == 2 * 2000
    a = np.lexsort((sr.positions[:, 2], sr.positions[:, 0]))
    np.testing.assert_array_equal(sr.positions[a][0::2], sr.positions[a][1::2])
    assert heat is not None and heat.water_heatmap.shape == (20, 20)


# ---- extensions: fixed-radius gather, Henyey-Greenstein phase ----------------------------


def _radius_cfg(name="replay_small.npz", R=0.5):
    import dataclasses

    return dataclasses.replace(config_from_fixture(load(name)), gather_radius=R)


def _hg_cfg(name="replay_small.npz", g=0.9):
    import dataclasses

    cfg = config_from_fixture(load(name))
    layers = tuple(dataclasses.replace(L, henyey_greenstein_g=g) for L in cfg.water.layers)
    return dataclasses.replace(cfg, water=dataclasses.replace(cfg.water, layers=layers))


# End to end, a record within ~1e-6 m of the radius can fall on either side of it when the
# tracer's float64 positions differ from the oracle's in the last bits, and one such record
# moves the waveform by its whole contribution (the k-NN estimate only swaps two nearly equal
# neighbours). Depth-profiled layers carry such last-bit differences (see the oracle's golden
# tests), so there the end-to-end bar is 1e-4; the gather itself is checked on identical
# inputs below.
@pytest.mark.parametrize("fixture,tol", [("replay_small.npz", REL_WAVEFORM_L1), ("replay_profiled.npz", 1e-4)])
def test_radius_gather_matches_oracle(gpu_available, fixture, tol):
    """Same Philox streams, fixed radius 0.5 m: GPU tracer + k-d radius traversal against
    the oracle's tracer + brute-force radius gather."""
    cfg = _radius_cfg(fixture)
    nf, nb, seed = 3000, 800, 43
    wf = _philox_run(cfg, nf, nb, seed, ids=False, precise=True)[2]
    orc = oracle_run(build_scene(cfg), nf, nb, seed=seed)
    assert orc["waveform"].sum() > 0
    for c in range(4):
        den = np.abs(orc["waveform"][c]).sum()
        if den:
            assert np.abs(wf[c] - orc["waveform"][c]).sum() / den < tol, c
        else:
            assert not wf[c].any(), c


@pytest.mark.parametrize("fixture", ["replay_small.npz", "replay_profiled.npz"])
def test_radius_gather_on_identical_inputs_matches_oracle(gpu_available, fixture):
    """The gather alone: the oracle's brute-force radius gather over the GPU's own exported
    maps and queries admits exactly the same records (float64 decision on identical float32
    map positions and hi+lo query positions), so the waveforms differ only by the float32
    arithmetic of each contribution: a few ulps for the planar channels; for the scatter
    channel the float32 phase-table bin weight (the same bar as the k-NN replay tests)."""
    from oracle.oracle import Oracle

    cfg = _radius_cfg(fixture)
    nf, nb, seed = 3000, 800, 47
    eng = _engine(cfg, ids=True, exits=False)
    try:
        eng.forward(nf, seed)
        maps = {c: eng.ctx.export_map(c) for c in range(4)}
        eng.build_maps()
        eng.backward(nb, seed)
        qs = {k: eng.ctx.export_queries(k) for k in range(3)}
        wf = eng.waveform_array(f64=True)
    finally:
        eng.close()
    orc = Oracle(build_scene(cfg))
    total = 0.0
    for ch, kind in ((0, 0), (1, 1), (2, 2), (3, 2)):
        pos, dr, e, t = maps[ch][:4]
        q = qs[kind]
        ref = np.zeros(wf.shape[1])
        if len(q["energy"]):
            orc.gather(ch, dict(pos=pos, dir=dr, energy=e, time=t),
                       dict(pos=q["pos"], dir=q["dir"].astype(np.float64), energy=q["energy"], time=q["time"]), ref)
        den = np.abs(ref).sum()
        total += den
        if den:
            assert np.abs(wf[ch] - ref).sum() / den < (REL_WAVEFORM_L1 if ch == 1 else 1e-6), ch
        else:
            assert not wf[ch].any(), ch
    assert total > 0


def test_radius_gather_bit_identical_run_to_run(gpu_available):
    cfg = _radius_cfg()
    a = _philox_run(cfg, 20000, 5000, 7, ids=False)[2]
    b = _philox_run(cfg, 20000, 5000, 7, ids=False)[2]
    np.testing.assert_array_equal(a, b)


def test_radius_gather_on_small_maps_needs_no_k(gpu_available):
    """The k-NN gather raises IndexError below k records; the fixed-radius gather has no
    such floor and matches the oracle on the same small maps."""
    cfg = _radius_cfg()
    fexit, maps, wf = _philox_run(cfg, 10, 200, 3, ids=False)
    orc = oracle_run(build_scene(cfg), 10, 200, seed=3)
    for c in range(4):
        den = np.abs(orc["waveform"][c]).sum()
        if den:
            assert np.abs(wf[c] - orc["waveform"][c]).sum() / den < REL_WAVEFORM_L1, c
        else:
            assert not wf[c].any(), c


def test_radius_gather_rk_reports_radius(gpu_available):
    cfg = _radius_cfg(R=0.25)
    eng = _engine(cfg, ids=True, exits=False)
    try:
        eng.forward(2000, 1)
        eng.build_maps()
        eng.backward(300, 1)
        q = eng.ctx.export_queries(1)
    finally:
        eng.close()
    assert len(q["rk"]) > 0
    np.testing.assert_array_equal(q["rk"], 0.25)


@pytest.mark.parametrize("fixture", ["replay_small.npz", "replay_profiled.npz"])
def test_philox_hg_matches_oracle(gpu_available, fixture):
    """Henyey-Greenstein phase (g = 0.9) through the phase-table path: the precise tracer
    and the oracle on the same Philox streams agree within the parity tolerance."""
    cfg = _hg_cfg(fixture)
    nf, nb = 3000, 800
    wf = _philox_run(cfg, nf, nb, 17, ids=False, precise=True)[2]
    orc = oracle_run(build_scene(cfg), nf, nb, seed=17)
    for c in range(4):
        den = np.abs(orc["waveform"][c]).sum()
        if den:
            assert np.abs(wf[c] - orc["waveform"][c]).sum() / den < REL_WAVEFORM_L1, c


def test_fast_and_precise_agree_in_distribution_hg(gpu_available):
    cfg = _hg_cfg("stats_small.npz")
    nf, nb = 60000, 15000
    tot = {}
    for precise in (True, False):
        tot[precise] = np.stack(
            [_philox_run(cfg, nf, nb, 900 + r, ids=False, precise=precise)[2].sum(1) / (nf * nb) for r in range(8)]
        )
    a, b = tot[True], tot[False]
    se = np.sqrt(a.var(0, ddof=1) / 8 + b.var(0, ddof=1) / 8)
    assert np.all(np.abs(a.mean(0) - b.mean(0)) < 4 * se + 1e-30), (a.mean(0), b.mean(0), se)


def _slope_cfg(sigma, name="replay_small.npz"):
    import dataclasses

    cfg = config_from_fixture(load(name))
    return dataclasses.replace(cfg, sea_surface=dataclasses.replace(cfg.sea_surface, slope_sigma=sigma))


def test_philox_slopes_match_oracle_photon_by_photon(gpu_available):
    """Gaussian surface slopes (extension): same facet draws on both sides, so records match
    the oracle photon by photon and the waveform within the parity tolerance."""
    cfg = _slope_cfg(0.1)
    nf, nb, seed = 4000, 1000, 77
    fexit, maps, wf = _philox_run(cfg, nf, nb, seed)
    orc = oracle_run(build_scene(cfg), nf, nb, seed=seed)
    for c in range(4):
        pos, dr, e, t, fwi, sfi, pid = maps[c]
        om = orc["maps"][c]
        assert len(e) == len(om["energy"]), c
        ia = np.lexsort((t, pid))
        ib = np.lexsort((om["time"], om["photon"]))
        np.testing.assert_array_equal(pid[ia], om["photon"][ib])
        np.testing.assert_array_equal(t[ia], om["time"][ib])
        np.testing.assert_allclose(pos[ia], om["pos"][ib], rtol=1e-5, atol=1e-5)
    for c in range(4):
        den = np.abs(orc["waveform"][c]).sum()
        if den:
            assert np.abs(wf[c] - orc["waveform"][c]).sum() / den < REL_WAVEFORM_L1, c


def test_fast_and_precise_agree_in_distribution_slopes(gpu_available):
    cfg = _slope_cfg(0.1, "stats_small.npz")
    nf, nb = 60000, 15000
    tot = {}
    for precise in (True, False):
        tot[precise] = np.stack(
            [_philox_run(cfg, nf, nb, 1300 + r, ids=False, precise=precise)[2].sum(1) / (nf * nb) for r in range(8)]
        )
    a, b = tot[True], tot[False]
    se = np.sqrt(a.var(0, ddof=1) / 8 + b.var(0, ddof=1) / 8)
    assert np.all(np.abs(a.mean(0) - b.mean(0)) < 4 * se + 1e-30), (a.mean(0), b.mean(0), se)


def test_slopes_refuse_replay(gpu_available):
    d = load("replay_small.npz")
    cfg = _slope_cfg(0.1)
    eng = _engine(cfg)
    try:
        with pytest.raises(ValueError):
            eng.forward(int(d["n_fwd"]), 0, replay=replay_streams(d, "fwd"))
    finally:
        eng.close()


@pytest.mark.gpu
def test_bench_geometry_replay_matches_reference(gpu_available):
    """Replay at the large scene's geometry (400 m, 20 m water, 420 000 integrator steps).
    A float32-ulp direction residual can move one crossing of a long path by a step, so up
    to 1% of photons may diverge; every other photon's map records and gather queries match
    the reference in step and energy (positions to 1 mm), and the waveform matches the
    reference's float64 accumulation and the oracle to 1e-4 in L1."""
    from fixtures import assert_same_records_except, diverged_photons

    d = load("replay_cfg1.npz")
    cfg = config_from_fixture(d)
    nf, nb = int(d["n_fwd"]), int(d["n_bwd"])
    eng = _engine(cfg)
    try:
        assert eng.scene.steps == int(d["steps"])
        eng.forward(nf, 0, replay=replay_streams(d, "fwd"))
        fexit = eng.ctx.exit_states(nf)
        maps = {c: eng.ctx.export_map(c) for c in range(4)}
        eng.build_maps()
        eng.backward(nb, 0, replay=replay_streams(d, "bwd"))
        bexit = eng.ctx.exit_states(nb)
        queries = {k: eng.ctx.export_queries(k) for k in range(3)}
        wf = eng.waveform_array(f64=True)
        scene = eng.scene
    finally:
        eng.close()
    fwd_div = set(np.nonzero(fexit["time"] != d["fwd_final_time"])[0].tolist())
    for c in range(4):
        pos, dr, e, t, fwi, sfi, pid = maps[c]
        if f"map{c}_pos" in d:
            fwd_div |= diverged_photons(pid, t, d[f"map{c}_ids"], d[f"map{c}_time"])
        else:
            assert len(e) == 0
    q = d["queries"]
    bwd_div = set(np.nonzero(bexit["time"] != d["bwd_final_time"])[0].tolist())
    for kind in range(3):
        ref = q[q[:, 0] == kind]
        bwd_div |= diverged_photons(queries[kind]["id"], queries[kind]["time"], ref[:, 1].astype(np.int64),
                                    ref[:, 9].astype(np.float32))
    assert len(fwd_div) <= 0.01 * nf and len(bwd_div) <= 0.01 * nb, (fwd_div, bwd_div)
    for c in range(4):
        if f"map{c}_pos" not in d:
            continue
        pos, dr, e, t, fwi, sfi, pid = maps[c]
        assert_same_records_except(dict(photon=pid, time=t, energy=e, pos=pos),
                                   dict(photon=d[f"map{c}_ids"], time=d[f"map{c}_time"],
                                        energy=d[f"map{c}_energy"], pos=d[f"map{c}_pos"]),
                                   fwd_div, atol_pos=1e-3)
    for kind in range(3):
        ref = q[q[:, 0] == kind]
        mine = queries[kind]
        assert_same_records_except(dict(photon=mine["id"], time=mine["time"], energy=mine["energy"], pos=mine["pos"]),
                                   dict(photon=ref[:, 1].astype(np.int64), time=ref[:, 9].astype(np.float32),
                                        energy=ref[:, 8], pos=ref[:, 2:5]),
                                   bwd_div, atol_pos=1e-3)
    orc = oracle_run(scene, nf, nb, replay_fwd=replay_streams(d, "fwd"), replay_bwd=replay_streams(d, "bwd"))
    for c in range(4):
        for ref in (d["waveform64"][c], orc["waveform"][c]):
            den = np.abs(ref).sum()
            if den:
                assert np.abs(wf[c] - ref).sum() / den < 1e-4, c


@pytest.mark.gpu
def test_stats_keep_the_forward_trace_counters(gpu_available):
    """The last forward trace's events and photons survive the backward trace (slots 28/29),
    so a step's interaction events are readable after it without a mid-step sync."""
    cfg = config_from_fixture(load("replay_small.npz"))
    eng = _engine(cfg, ids=False, exits=False, precise=False)
    try:
        eng.forward(4000, 11)
        fwd = eng.ctx.stats()
        eng.build_maps()
        eng.backward(1000, 11)
        st = eng.ctx.stats()
    finally:
        eng.close()
    # every photon meets the surface at least once inside the window
    assert fwd["photons"] == 4000 and fwd["events"] >= 4000
    assert st["forward_events"] == fwd["events"] and st["forward_photons"] == 4000
    assert st["photons"] == 1000 and st["events"] >= 1000
