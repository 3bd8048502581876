"""Pin the oracle (CPU restatement) to the reference: replayed runs against the reference's
recorded runs, k-NN against scipy's KDTree answers, Philox statistics against independent
reference runs. These run on the CPU only."""

import numpy as np
import pytest

from fixtures import assert_statistically_equal, config_from_fixture, load, replay_streams
from oracle.oracle import Oracle, oracle_run
from pyalbsim_gb300.scene import build_scene

REPLAYS = ["small", "twolayer", "cfg0", "profiled"]


@pytest.fixture(scope="module", params=REPLAYS)
def replayed(request):
    d = load(f"replay_{request.param}.npz")
    scene = build_scene(config_from_fixture(d))
    r = oracle_run(scene, int(d["n_fwd"]), int(d["n_bwd"]),
                   replay_fwd=replay_streams(d, "fwd"), replay_bwd=replay_streams(d, "bwd"))
    return request.param, d, scene, r


def test_steps_match(replayed):
    _, d, scene, _ = replayed
    assert scene.steps == int(d["steps"])


def _assert_energy(d, mine, ref):
    """Energies are bit-exact for constant layers. In depth-profiled layers the albedo
    depends continuously on the float64 position, whose last bits differ from NumPy's
    vectorised kernels (norms, exp/log); a flipped float32 rounding of the albedo then
    shows as a one-ulp energy difference, so there the bar is the 1e-5 parity tolerance."""
    prof = d.get("cfg_layer_prof")
    if prof is not None and np.any(prof[:, :, 0] != 0):
        np.testing.assert_allclose(mine, ref, rtol=1e-5, atol=0)
    else:
        np.testing.assert_array_equal(mine, ref)


def test_photon_maps_record_by_record(replayed):
    """Same records (photon, step) per type; energies and times exact; geometry to 1e-6."""
    _, d, _, r = replayed
    for c in range(4):
        mp = r["maps"][c]
        if f"map{c}_pos" not in d:
            assert len(mp["energy"]) == 0
            continue
        ia = np.lexsort((mp["time"], mp["photon"]))
        ib = np.lexsort((d[f"map{c}_time"], d[f"map{c}_ids"]))
        np.testing.assert_array_equal(mp["photon"][ia], d[f"map{c}_ids"][ib])
        np.testing.assert_array_equal(mp["time"][ia], d[f"map{c}_time"][ib])
        _assert_energy(d, mp["energy"][ia], d[f"map{c}_energy"][ib])
        np.testing.assert_allclose(mp["pos"][ia], d[f"map{c}_pos"][ib], rtol=1e-6, atol=1e-5)
        np.testing.assert_allclose(mp["dir"][ia], d[f"map{c}_dir"][ib], rtol=0, atol=1e-6)
        fa, fb = mp["fwi"][ia], d[f"map{c}_fwi"][ib]
        np.testing.assert_array_equal(np.isnan(fa), np.isnan(fb))
        np.testing.assert_allclose(fa[~np.isnan(fa)], fb[~np.isnan(fb)], rtol=1e-6, atol=1e-5)


def test_exit_states(replayed):
    _, d, _, r = replayed
    for p in ("fwd", "bwd"):
        ex = r[f"{p}_exit"]
        _assert_energy(d, ex["energy"], d[f"{p}_final_energy"])
        np.testing.assert_array_equal(ex["tau_target"], d[f"{p}_final_tau_target"])
        np.testing.assert_array_equal(ex["time"], d[f"{p}_final_time"])
        np.testing.assert_allclose(ex["tau"], d[f"{p}_final_tau"], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(ex["pos"], d[f"{p}_final_pos"], rtol=1e-5, atol=1e-4)
        np.testing.assert_allclose(ex["dir"], d[f"{p}_final_dir"], rtol=0, atol=1e-5)


def test_waveform_float64(replayed):
    """Float64-accumulated reference waveform: L1 within 1e-6 per channel."""
    _, d, _, r = replayed
    for c in range(4):
        ref = d["waveform64"][c]
        got = r["waveform"][c]
        den = np.abs(ref).sum()
        if den == 0:
            assert np.abs(got).sum() == 0
            continue
        assert np.abs(got - ref).sum() / den < 1e-6, c


def test_waveform_float32_reference_units(replayed):
    """The reference's own float32 accumulation, within its rounding error."""
    _, d, _, r = replayed
    for c in range(4):
        ref = d["waveform32"][c].astype(np.float64)
        den = np.abs(ref).sum()
        if den:
            assert np.abs(r["waveform"][c] - ref).sum() / den < 1e-4


def test_queries(replayed):
    """Backward events (gather queries) match the reference's event by event. The reference
    logs a surface entry twice (SURFACE_REFLECTION and SURFACE_TRANSMISSION_UP gathers);
    query kind 0/1/2 corresponds to its channel 0/1/2 entries."""
    _, d, _, r = replayed
    q = d["queries"]  # channel, photon, pos3, dir3, E, t, contribution sum
    for kind in range(3):
        mine = r["queries"][kind]
        ref = q[q[:, 0] == kind]
        if len(ref) == 0:
            assert len(mine["energy"]) == 0
            continue
        ia = np.lexsort((mine["time"], mine["photon"]))
        ib = np.lexsort((ref[:, 9], ref[:, 1]))
        np.testing.assert_array_equal(mine["photon"][ia], ref[ib, 1].astype(np.int64))
        np.testing.assert_array_equal(mine["time"][ia], ref[ib, 9].astype(np.float32))
        np.testing.assert_allclose(mine["pos"][ia], ref[ib, 2:5], rtol=1e-6, atol=1e-5)
        _assert_energy(d, mine["energy"][ia], ref[ib, 8].astype(np.float32))


def test_heatmaps(replayed):
    name, d, _, r = replayed
    if "heat_radius" not in d:
        return
    np.testing.assert_array_equal(r["heat_radius"].reshape(d["heat_radius"].shape), d["heat_radius"].astype(np.uint32))
    for key, mine in (("heat_water", r["heat_water"]), ("heat_floor", r["heat_floor"])):
        ref = d[key].astype(np.float64).ravel()
        den = np.abs(ref).sum()
        assert np.abs(mine - ref).sum() / den < 1e-4, key


def test_knn_matches_kdtree():
    kn = load("knn.npz")
    for name in ("planar", "cloud", "cloud_k16"):
        pts, qs, k = kn[f"{name}_points"], kn[f"{name}_queries"], int(kn[f"{name}_k"])
        orc = Oracle(build_scene(config_from_fixture(load("replay_small.npz"))))
        dist, idx = orc.knn(pts, qs, k)
        np.testing.assert_allclose(dist, kn[f"{name}_dist"], rtol=1e-12, atol=0)
        for i in range(len(qs)):
            ref = kn[f"{name}_idx"][i]
            rd = kn[f"{name}_dist"][i]
            # sets must agree except for exact ties at the k-th distance
            strict = set(ref[rd < rd[-1]])
            assert strict <= set(idx[i]), (name, i)


def test_oracle_philox_statistics_match_reference():
    """Philox runs of the oracle agree with independent reference runs per waveform bin
    within 3 combined standard errors, and in normalised L1 within the MC noise."""
    st = load("stats_small.npz")
    scene = build_scene(config_from_fixture(st))
    runs, nf, nb = 32, int(st["n_fwd"]), int(st["n_bwd"])
    waves = []
    for r in range(runs):
        out = oracle_run(scene, nf, nb, seed=777 + r)
        waves.append(out["waveform"] / (nf * nb))
    w = np.stack(waves)
    assert_statistically_equal(w, st)



def test_bench_geometry_replay_matches_reference_photon_by_photon():
    """The large scene's geometry (400 m, 20 m water, 0.05 ns bins: 420 000 integrator
    steps). Over paths this long, a direction that differs from NumPy's vectorised kernels
    by a float32 ulp (the residual of the other replays) can move one plane or
    optical-depth crossing by a step; that photon then diverges. At most 1% of photons may
    do so. Every other photon's map records and gather queries match in step and energy
    (positions to 1 mm), and the waveform matches the reference's float64 accumulation to 1e-4 in L1."""
    from fixtures import assert_same_records_except, diverged_photons

    d = load("replay_cfg1.npz")
    scene = build_scene(config_from_fixture(d))
    assert scene.steps == int(d["steps"])
    nf, nb = int(d["n_fwd"]), int(d["n_bwd"])
    r = oracle_run(scene, nf, nb, replay_fwd=replay_streams(d, "fwd"), replay_bwd=replay_streams(d, "bwd"))
    fwd_div = set()
    for c in range(4):
        mp = r["maps"][c]
        if f"map{c}_pos" in d:
            fwd_div |= diverged_photons(mp["photon"], mp["time"], d[f"map{c}_ids"], d[f"map{c}_time"])
    fwd_div |= set(np.nonzero(r["fwd_exit"]["time"] != d["fwd_final_time"])[0].tolist())
    q = d["queries"]
    bwd_div = set(np.nonzero(r["bwd_exit"]["time"] != d["bwd_final_time"])[0].tolist())
    for kind in range(3):
        ref = q[q[:, 0] == kind]
        mine = r["queries"][kind]
        bwd_div |= diverged_photons(mine["photon"], mine["time"], ref[:, 1].astype(np.int64),
                                    ref[:, 9].astype(np.float32))
    assert len(fwd_div) <= 0.01 * nf and len(bwd_div) <= 0.01 * nb, (fwd_div, bwd_div)
    for c in range(4):
        if f"map{c}_pos" not in d:
            continue
        mp = r["maps"][c]
        ref = dict(photon=d[f"map{c}_ids"], time=d[f"map{c}_time"], energy=d[f"map{c}_energy"],
                   pos=d[f"map{c}_pos"])
        # over ~100 m of path a float32-ulp direction difference moves a position by < 1 mm
        assert_same_records_except(dict(photon=mp["photon"], time=mp["time"], energy=mp["energy"], pos=mp["pos"]),
                                   ref, fwd_div, atol_pos=1e-3)
    for kind in range(3):
        ref = q[q[:, 0] == kind]
        mine = r["queries"][kind]
        assert_same_records_except(mine, dict(photon=ref[:, 1].astype(np.int64), time=ref[:, 9].astype(np.float32),
                                              energy=ref[:, 8], pos=ref[:, 2:5]), bwd_div, atol_pos=1e-3)
    for c in range(4):
        ref = d["waveform64"][c]
        den = np.abs(ref).sum()
        if den:
            assert np.abs(r["waveform"][c] - ref).sum() / den < 1e-4, c


def test_oracle_edge_cases_zero_photons_and_empty_maps():
    """No photons trace to an all-zero waveform; backward photons against empty maps, or
    maps with fewer than k records, raise IndexError (the reference's KDTree quirk)."""
    cfg = config_from_fixture(load("replay_small.npz"))
    scene = build_scene(cfg)
    assert not oracle_run(scene, 0, 0, seed=1)["waveform"].any()
    assert not oracle_run(scene, 50, 0, seed=1)["waveform"].any()
    for nf in (0, 5):
        with pytest.raises(IndexError):
            oracle_run(scene, nf, 10, seed=1)
