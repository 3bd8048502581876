"""Known-answer tests of the host-side scene model and the oracle's physics functions
against values the reference's own functions returned (tests/golden/kat_physics.npz)."""

import numpy as np
import pytest

from fixtures import config_from_fixture, load
from pyalbsim_gb300.config import (
    HeatmapConfig, LaserConfig, SceneConfig, SeaFloorConfig, SeaSurfaceConfig, SensorConfig,
    SimulationConfig, TurbidityLayerConfig, WaterConfig,
)
from pyalbsim_gb300.scene import (
    build_scene, fournier_forand_backscatter, fournier_forand_table, refract, rotation_z_to,
)

KAT = load("kat_physics.npz")


def small_config():
    return SimulationConfig(
        photon_mapping_k=32,
        scene=SceneConfig(flying_height=10.0),
        water=WaterConfig(layers=(TurbidityLayerConfig(
            height=2.0, absorption_coefficient=0.1, scattering_coefficient=1.0, refractive_index=1.34),)),
        laser=LaserConfig(divergence_angle=5e-3, nadir_angle=10.0, azimuth_angle=30.0, pulse_fwhm=3e-9),
        sensor=SensorConfig(aperture_radius=0.1, field_of_view=50e-3, sample_rate=int(1e9)),
        sea_floor=SeaFloorConfig(albedo=0.2),
        sea_surface=SeaSurfaceConfig(albedo=0.1, roughness=float(np.sqrt(0.05))),
        heatmap=HeatmapConfig(enabled=True, bins=20, water_extent=1.0, seafloor_extent=3.0),
    )


def two_layer_config():
    return SimulationConfig(
        photon_mapping_k=24,
        scene=SceneConfig(flying_height=8.0),
        water=WaterConfig(layers=(
            TurbidityLayerConfig(height=0.7, absorption_coefficient=0.2, scattering_coefficient=1.5),
            TurbidityLayerConfig(height=1.3, absorption_coefficient=0.05, scattering_coefficient=0.6,
                                 refractive_index=1.36),
        )),
        laser=LaserConfig(divergence_angle=4e-3, nadir_angle=0.0, pulse_fwhm=3e-9),
        sensor=SensorConfig(aperture_radius=0.05, field_of_view=40e-3, sample_rate=int(1e9)),
        sea_floor=SeaFloorConfig(albedo=0.3),
        heatmap=HeatmapConfig(enabled=False),
    )


def config0_geometry():
    return SimulationConfig(
        scene=SceneConfig(flying_height=400.0),
        water=WaterConfig(layers=(TurbidityLayerConfig(
            height=5.0, absorption_coefficient=0.05, scattering_coefficient=0.20, refractive_index=1.34),)),
        laser=LaserConfig(divergence_angle=1e-3, nadir_angle=0.0, pulse_fwhm=3e-9),
        sensor=SensorConfig(field_of_view=20e-3, sample_rate=int(1e10)),
        sea_floor=SeaFloorConfig(albedo=0.15),
        sea_surface=SeaSurfaceConfig(roughness=float(np.sqrt(0.05))),
        heatmap=HeatmapConfig(enabled=False),
    )


CONFIGS = [small_config, two_layer_config, config0_geometry, SimulationConfig]


def test_fournier_forand_tables_bit_exact():
    for i in range(3):
        junge, nratio = KAT[f"ff{i}_params"]
        stride = int(KAT[f"ff{i}_stride"])
        _, pf, cdf = fournier_forand_table(junge, nratio)
        np.testing.assert_array_equal(pf[::stride], KAT[f"ff{i}_pf"])
        np.testing.assert_array_equal(cdf[::stride], KAT[f"ff{i}_cdf"])
        assert fournier_forand_backscatter(junge, nratio) == KAT[f"ff{i}_bb"]


def test_model_scalars_match_reference():
    rows = KAT["model_rows"]
    for row in rows:
        ci, li = int(row[0]), int(row[1])
        s = build_scene(CONFIGS[ci]())
        layer = s.layers[li]
        assert s.steps == int(row[2])
        assert s.dt == row[3]
        assert s.surface_y == row[4] and s.floor_y == row[5]
        assert layer.alpha64 == row[6]                      # Churnside lidar attenuation
        assert layer.ssa32 == np.float32(row[7])            # single-scattering albedo (float32 store)
        assert layer.speed32 == float(np.float32(row[8]))   # c / n stored as float32
        assert s.f0 == row[9]
        np.testing.assert_array_equal(s.laser_dir, row[10:13])
        np.testing.assert_allclose(s.water_center, row[13:16], rtol=0, atol=1e-12)
        np.testing.assert_allclose(s.floor_center, row[16:19], rtol=0, atol=1e-12)


def test_rotation_matrices_bit_exact():
    for v, r in zip(KAT["rot_in"], KAT["rot_out"]):
        np.testing.assert_array_equal(rotation_z_to(v), r)


def test_snell_refraction():
    for tag, sgn in (("up", 1), ("down", -1)):
        for d, t, tir in zip(KAT[f"snell_in_{tag}"], KAT[f"snell_out_{tag}"], KAT[f"snell_tir_{tag}"]):
            out, flag = refract(d, np.array([0.0, sgn, 0.0]), 1.0, 1.34)
            np.testing.assert_allclose(out, t, rtol=0, atol=2e-16)
            assert flag == tir


def test_ggx_reflected_energy_oracle():
    from oracle.oracle import kat_ggx

    for r_i, rough in enumerate(KAT["ggx_rough"]):
        for w_i, wo in enumerate(KAT["ggx_wo"]):
            ref = KAT[f"ggx_{r_i}_{w_i}"]
            got = kat_ggx(rough, 0.0211, KAT["ggx_wi"], wo)
            np.testing.assert_allclose(got, ref, rtol=2e-7, atol=1e-30)


def test_scatter_bin_energy_oracle():
    from oracle.oracle import kat_scatter_energy

    s = build_scene(small_config())  # FF(3.62, 1.1) tables, as the fixture
    # the fixture passed its vector as calculate_energy_batch's view direction
    got = kat_scatter_energy(s, KAT["senergy_pdirs"], KAT["senergy_sdir"])
    np.testing.assert_allclose(got, KAT["senergy_val"], rtol=1e-12, atol=0)


@pytest.mark.parametrize("mk", CONFIGS)
def test_scene_struct_packs(mk):
    from pyalbsim_gb300._native import scene_struct

    s = build_scene(mk())
    p, keep = scene_struct(s)
    assert p.n_layers == len(s.layers)
    assert p.steps == s.steps and p.k == s.k
    assert abs(p.layers[p.n_layers - 1].bottom_depth - s.depth) < 1e-12


def test_profiled_attenuation_lut_matches_reference():
    """Depth-profiled layers: the attenuation LUT (float32 depths, float64 values) equals the
    reference's TurbidityLayerModel LUT bit for bit (linear and exponential IOPs, a linear
    salinity profile)."""
    d = load("replay_profiled.npz")
    scene = build_scene(config_from_fixture(d))
    n = 0
    for i, layer in enumerate(scene.layers):
        if f"lut{i}_z" not in d:
            assert layer.constant
            continue
        n += 1
        assert not layer.constant
        np.testing.assert_array_equal(layer.lut_z, d[f"lut{i}_z"])
        np.testing.assert_array_equal(layer.lut_alpha, d[f"lut{i}_alpha"])
    assert n == 2


def test_fast_tracer_free_paths_at_the_bench_geometry():
    """The float32 tracer takes ceil((tau* - tau) / inc) steps to the next scatter, while the
    reference accumulates tau <- fl32(fl64(tau) + inc) step by step, whose rounding is a
    fixed fraction of an ulp inside each binade of tau. At the large scene's attenuation and
    step length (inc ~ 4.9e-4) the two step counts agree to 1e-4 in the mean over
    exponential tau* (measured 1.5e-5 at 2e5 samples), far below one integrator step over a
    20 m path."""
    from pyalbsim_gb300.workloads import large

    sc = build_scene(large())
    L = sc.layers[0]
    inc = np.float32(np.float32(L.alpha32) * np.float32(np.float32(L.speed32) * np.float32(sc.dt)))
    rng = np.random.default_rng(1)
    taut = (-np.log(rng.random(20000).astype(np.float32))).astype(np.float32)
    tau = np.zeros_like(taut)
    steps = np.zeros(len(taut), np.int64)
    active = np.ones(len(taut), bool)
    for _ in range(200000):
        if not active.any():
            break
        tau[active] = (tau[active].astype(np.float64) + np.float64(inc)).astype(np.float32)
        steps[active] += 1
        active &= ~(tau >= taut)
    assert not active.any()
    closed = np.maximum(np.ceil(taut.astype(np.float64) / np.float64(inc)).astype(np.int64), 1)
    assert abs(steps.sum() / closed.sum() - 1.0) < 1e-4
    assert np.abs(steps - closed).max() <= 0.005 * closed.max()


def test_fast_tracer_inverse_cdf_table_resolution():
    """The float32 tracer draws the scattering angle from theta(u) tabulated at u = j/65536
    (numpy.interp on the phase CDF, as the context builds it) and interpolated linearly;
    the precise tracer interpolates the 18 000-angle CDF itself. At the large scene's FF
    phase function the two agree to ~1e-7 rad on average; only the flat backscatter end of
    the CDF (u -> 1) leaves differences above 1e-4 rad, on < 1e-3 of the draws."""
    from pyalbsim_gb300.workloads import large

    L = build_scene(large()).layers[0]
    th = np.asarray(L.ff_theta, np.float64)
    cdf = np.asarray(L.ff_cdf, np.float64)
    K = 65536
    inv = np.interp(np.arange(K + 1) / K, cdf, th).astype(np.float32)
    u = (np.random.default_rng(0).integers(0, 2**23, 400000) + 0.5) / 2**23  # the fast tracer's uniforms
    exact = np.interp(u, cdf, th)
    x = u * K
    j = np.minimum(x.astype(np.int64), K - 1)
    fast = inv[j] + (x - j) * (inv[j + 1] - inv[j])
    d = np.abs(fast - exact)
    assert d.mean() < 1e-6
    assert (d > 1e-4).mean() < 1e-3
    assert abs(np.cos(fast).mean() - np.cos(exact).mean()) < 1e-7
