"""Host-side scene model: every constant and table the device kernels consume.

This restates, in float64 NumPy, the parts of the reference model that are evaluated once
per configuration:

* time step and step count (``alb_sim/physics/models/simulation.py:35-49``);
* laser axis from DEGREES (``alb_sim/physics/models/laser.py:22-33``) and the float32
  Rodrigues matrix that rotates +z onto it (``alb_sim/math/rotation_matrix.py:39-102``);
* Fournier-Forand phase table and CDF on 18000 angles and the backscatter fraction
  (``alb_sim/physics/scatter/fournier_forand_phase_function.py:9-48, 89-111``);
* Churnside lidar attenuation alpha and single-scattering albedo (alpha - a) / alpha
  (``alb_sim/physics/models/water.py:117-184, 237-245``);
* Schlick base reflectance from the top layer's refractive index
  (``alb_sim/physics/models/sea_surface.py:30-33``);
* the per-angular-bin scatter weight table used by the gather
  (``alb_sim/physics/scatter/energy.py:8-52``).

Any object exposing the reference's config attribute names is accepted, so the
reference's own ``SimulationConfig`` instances work unchanged.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

LIGHT_SPEED_AIR = 2.998e8
FLOAT32_EPS = float(np.finfo(np.float32).eps)
SCATTER_DIVISIONS = 18000

CH_BOTTOM, CH_SCATTER, CH_SURFACE_REFLECTION, CH_SURFACE_TRANSMISSION_UP = 0, 1, 2, 3
MAX_LAYERS = 8


def fournier_forand_table(junge_slope: float, n_ratio: float):
    """FF phase function p(theta) on 18000 angles in [1e-6, pi] and its normalised CDF.

    The CDF is the running sum of p(theta) * sin(theta) divided by its last element.
    """
    theta = np.linspace(1e-6, np.pi, SCATTER_DIVISIONS, dtype=np.float64)
    nu = (3.0 - junge_slope) / 2.0
    k = 4.0 / (3.0 * (n_ratio - 1.0) ** 2)
    s2 = np.sin(theta / 2.0) ** 2
    dl = k * s2
    d180 = k * np.sin(np.pi / 2.0) ** 2
    dl_nu = dl**nu
    main = (
        nu * (1.0 - dl)
        - (1.0 - dl_nu)
        + (dl * (1.0 - dl_nu) - nu * (1.0 - dl)) * np.sin(theta / 2.0) ** (-2)
    ) * (1.0 / (4.0 * np.pi * (1.0 - dl) ** 2 * dl_nu))
    back = ((1.0 - d180**nu) / (16.0 * np.pi * (d180 - 1.0) * d180**nu)) * (
        3.0 * np.cos(theta) ** 2 - 1.0
    )
    pf = main + back
    cdf = np.cumsum(pf * np.sin(theta))
    cdf /= cdf[-1]
    return theta, pf, cdf


def henyey_greenstein_table(g: float):
    """Henyey-Greenstein p(theta) = (1 - g^2) / (4 pi (1 + g^2 - 2 g cos theta)^1.5) on the FF
    angle grid, with the CDF formed the same way (running sum of p sin theta, normalised), so
    the sampling tables and the gather's bin weights follow the phase-table path unchanged."""
    theta = np.linspace(1e-6, np.pi, SCATTER_DIVISIONS, dtype=np.float64)
    pf = (1.0 - g * g) / (4.0 * np.pi * (1.0 + g * g - 2.0 * g * np.cos(theta)) ** 1.5)
    cdf = np.cumsum(pf * np.sin(theta))
    cdf /= cdf[-1]
    return theta, pf, cdf


def henyey_greenstein_backscatter(g: float) -> np.float64:
    """Backward-hemisphere fraction of HG: (1 - g) / (2 g) ((1 + g) / sqrt(1 + g^2) - 1)."""
    return np.float64((1.0 - g) / (2.0 * g) * ((1.0 + g) / np.sqrt(1.0 + g * g) - 1.0))


def fournier_forand_backscatter(junge_slope: float, n_ratio: float) -> float:
    """Fraction of FF scattering into the backward hemisphere (closed form at 90 deg)."""
    nu = (3.0 - junge_slope) / 2.0
    d90 = (4.0 / (3.0 * (n_ratio - 1.0) ** 2)) * np.sin(np.pi / 4.0) ** 2
    top = 1.0 - d90 ** (nu + 1.0) - 0.5 * (1.0 - d90**nu)
    bottom = (1.0 - d90) * d90**nu
    return float(1.0 - top / bottom)


def churnside_alpha(a, b, salinity, wavelength_um, flying_height, divergence, bb_frac):
    """Lidar attenuation coefficient alpha (1/m) of a homogeneous water parcel.

    alpha = Kd + (b_p - 4.18 b_p B (1 - 0.52 e^{-10.8 b})) exp(-0.85 D (a + b_p)),
    Kd = a + 4.18 b_p B (1 - 0.52 e^{-10.8 a}), b_p = b - b_w(salinity, lambda),
    D = 2 H tan(div / 2) the laser spot diameter at the surface.
    """
    b_w = (1.0 + 0.008027 * salinity) * 0.00012 * wavelength_um ** (-4.24)
    b_p = b - b_w
    spot = 2.0 * flying_height * math.tan(divergence / 2.0)
    kd = a + 4.18 * b_p * bb_frac * (1.0 - 0.52 * np.exp(-10.8 * a))
    beam_part = (b_p - 4.18 * b_p * bb_frac * (1.0 - 0.52 * np.exp(-10.8 * b))) * np.exp(
        -0.85 * spot * (a + b_p)
    )
    return kd + beam_part


def rotation_z_to(v) -> np.ndarray:
    """float32 matrix rotating +z onto the direction ``v`` (Rodrigues, with the
    reference's isclose() special cases for +z and -z)."""
    v = np.asarray(v, dtype=np.float64)
    v = v / np.linalg.norm(v)
    c = v[2]
    ax, ay = -v[1], v[0]
    if np.isclose(c, 1.0):
        return np.eye(3, dtype=np.float32)
    if np.isclose(c, -1.0):
        return np.array([[1, 0, 0], [0, -1, 0], [0, 0, -1]], dtype=np.float32)
    s2 = ax * ax + ay * ay
    K = np.array([[0.0, 0.0, ay], [0.0, 0.0, -ax], [-ay, ax, 0.0]])
    R = np.eye(3) + K + (K @ K) * ((1.0 - c) / s2)
    return R.astype(np.float32)


def scatter_weight_table(theta: np.ndarray, cdf: np.ndarray):
    """Gather weight per angular bin: CDF mass of bin i of width (pi - eps32) / 18000.

    The bin width is a float32 quantity in the reference (numpy scalar promotion), so it
    is kept as float32 here and the bin edges are i * width in float64.
    """
    n = len(theta)
    width32 = np.float32(np.float32(np.pi) - np.float32(FLOAT32_EPS)) / np.float32(n)
    width = float(width32)
    i = np.arange(n, dtype=np.float64)
    lo = np.interp(i * width, theta, cdf)
    hi = np.interp((i + 1.0) * width, theta, cdf)
    return (hi - lo), width32


def _is_constant(layer) -> bool:
    return all(
        isinstance(getattr(layer, name), float)
        for name in (
            "scattering_coefficient",
            "absorption_coefficient",
            "salinity",
            "refractive_index",
        )
    )


def _value_at(value, z_local, height):
    if isinstance(value, float):
        return value
    return value.at(z_local / height)


def _profile_code(value):
    """(kind, start, end) of a layer property: 0 constant, 1 linear, 2 exponential."""
    if isinstance(value, float):
        return (0, float(value), float(value))
    name = type(value).__name__
    if name == "LinearParameter":
        return (1, float(value.start), float(value.end))
    if name == "ExponentialParameter":
        return (2, float(value.start), float(value.end))
    raise ValueError(f"unsupported depth profile {name}: LinearParameter or ExponentialParameter expected")


def attenuation_lut(layer, wavelength, flying_height, divergence, bb_frac):
    """The reference's attenuation LUT of a profiled layer
    (TurbidityLayerModel._build_lidar_attenuation_lut, water.py:85-101): the Churnside
    coefficient at num_sublayers float32 local depths, profiles evaluated at z / height with
    the profiles' own float32 / float64 arithmetic."""
    z = np.linspace(0.0, layer.height, int(layer.num_sublayers), dtype=np.float32)
    a = _value_at(layer.absorption_coefficient, z, layer.height)
    b = _value_at(layer.scattering_coefficient, z, layer.height)
    s = _value_at(layer.salinity, z, layer.height)
    # the reference's backscatter fraction is a NumPy float64 scalar, which (unlike a Python
    # float) promotes float32 profile arrays to float64 in the formula
    alpha = churnside_alpha(a, b, s, wavelength, flying_height, divergence, np.float64(bb_frac))
    return z, np.asarray(alpha)


@dataclass
class LayerModel:
    height: float
    bottom_depth: float  # cumulative depth of the layer's lower boundary
    constant: bool
    alpha64: float  # lidar attenuation at the layer top (constant layers: everywhere)
    alpha32: float  # float32-rounded, the value the integrator adds up
    ssa32: float  # single-scattering albedo, float32
    speed32: float  # c / n rounded to float32 (the reference stores speeds in float32)
    n_top: float
    absorption: float
    ff_theta: np.ndarray
    ff_cdf: np.ndarray
    ff_slope: np.ndarray
    backscatter: float
    scatter_weight: np.ndarray
    bin_width32: float
    top32: float = 0.0  # depth of the layer top, float32 (the reference's layer offset z0)
    # depth profiles (profiled layers only): attenuation LUT on float32 local depths and
    # the (kind, start, end) of the refractive index and absorption profiles
    lut_z: Optional[np.ndarray] = None
    lut_alpha: Optional[np.ndarray] = None
    n_profile: Tuple[int, float, float] = (0, 0.0, 0.0)
    a_profile: Tuple[int, float, float] = (0, 0.0, 0.0)
    # adjoint (extension): d ln(alpha)/d theta and d ln(ssa)/d theta for theta = (a, b, g),
    # the HG asymmetry (0: Fournier-Forand layer) and d ln(scatter weight)/dg per bin
    dlog_alpha: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    dlog_ssa: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    hg_g: float = 0.0
    dlog_weight_g: Optional[np.ndarray] = None
    # d ln(mass)/dg of each interval of the HG sampling table (the exact score of a drawn angle)
    dlog_sample_g: Optional[np.ndarray] = None


_CSTEP = 1e-30  # complex-step size: f'(x) = Im f(x + i h) / h, exact to rounding


def adjoint_layer_terms(a, b, salinity, wavelength, flying_height, divergence, bb_frac, hg_g=None):
    """d ln(alpha)/d theta and d ln(ssa)/d theta for theta = (a, b, g) of a constant layer,
    by complex-step differentiation of the Churnside attenuation and ssa = (alpha - a)/alpha;
    with hg_g set, g moves the backscatter fraction B of an HG layer (for a Fournier-Forand
    layer the g entries are 0)."""

    def alpha_ssa(da=0.0, db=0.0, dg=0.0):
        bb = bb_frac if hg_g is None else _hg_backscatter(hg_g + dg)
        al = churnside_alpha(a + da, b + db, salinity, wavelength, flying_height, divergence, bb)
        return al, (al - (a + da)) / al

    al0, ssa0 = alpha_ssa()
    al0, ssa0 = float(np.real(al0)), float(np.real(ssa0))
    dla, dls = [], []
    for i in range(3):
        if i == 2 and hg_g is None:
            dla.append(0.0)
            dls.append(0.0)
            continue
        kw = {("da", "db", "dg")[i]: 1j * _CSTEP}
        al, ssa = alpha_ssa(**kw)
        dla.append(float(np.imag(al)) / _CSTEP / al0)
        dls.append(float(np.imag(ssa)) / _CSTEP / ssa0)
    return tuple(dla), tuple(dls)


def _hg_backscatter(g):
    return (1.0 - g) / (2.0 * g) * ((1.0 + g) / np.sqrt(1.0 + g * g) - 1.0)


def hg_weight_dlog_g(g: float, weight: np.ndarray) -> np.ndarray:
    """d ln(scatter weight)/dg per angular bin of an HG layer. The weight is the CDF mass of
    each bin, linear in the CDF on a fixed angle grid, so its derivative is the same bin
    mass of dCDF/dg (complex step through the normalised running sum)."""
    th, _, cdf_c = henyey_greenstein_table(g + 1j * _CSTEP)
    dcdf = np.imag(cdf_c) / _CSTEP
    dw, _ = scatter_weight_table(th, dcdf)
    out = np.zeros_like(weight, dtype=np.float64)
    np.divide(dw, weight, out=out, where=weight > 0)
    return out


def hg_sample_dlog_g(g: float) -> np.ndarray:
    """Score of an HG scattering angle as the tracers draw it: d ln(mass)/dg of the table
    interval it falls in. Inverting the tabulated CDF (linear between grid angles) puts the
    angle in interval i, (theta_{i-1}, theta_i], with probability C_i - C_{i-1}, uniformly
    within it (i = 0: theta_0 with probability C_0), so the log-density of the drawn angle
    moves with g exactly as that interval's mass does. The analytic d ln p_HG(mu)/dg is not the
    score of this distribution: when the HG peak is narrow against the grid (g = 0.99: width
    ~0.01 rad, grid step 1.75e-4 rad) its mean under the table is +0.70 per scatter instead of
    0 (+0.007 at g = 0.9). Complex step through the normalised running sum."""
    _, _, cdf_c = henyey_greenstein_table(g + 1j * _CSTEP)
    mass = np.diff(np.concatenate(([0.0 + 0.0j], cdf_c)))
    out = np.zeros(len(mass), dtype=np.float64)
    np.divide(np.imag(mass) / _CSTEP, np.real(mass), out=out, where=np.real(mass) > 0)
    return out


@dataclass
class SceneModel:
    """Everything derived from a configuration; the source of the C ABI scene struct."""

    sample_rate: int
    sample_multiplier: int
    k: int
    dt: float
    steps: int
    total_substeps: int
    surface_y: float
    floor_y: float
    depth: float
    laser_dir: np.ndarray
    laser_rot32: np.ndarray
    divergence: float
    fov: float
    aperture_radius: float
    pulse_sigma: float
    effective_rate: float
    n_water: float
    f0: float
    seafloor_albedo: float
    surface_albedo: float
    roughness: float
    flying_height: float
    layers: List[LayerModel] = field(default_factory=list)
    heatmap_enabled: bool = False
    gather_radius: Optional[float] = None  # extension: fixed-radius gather (m), None = k-NN
    heatmap_bins: int = 200
    heatmap_water_extent: float = 1.0
    heatmap_seafloor_extent: float = 10.0
    water_center: np.ndarray = None
    floor_center: np.ndarray = None
    # extension: gated waveform window [gate_start, gate_start + gate_bins) of the timeline
    gate_start: int = 0
    gate_bins: int = 0
    slope_sigma: float = 0.0  # extension: Gaussian surface-slope std (0 = flat)

    @property
    def n_bins(self) -> int:
        return self.gate_bins if self.gate_bins > 0 else 2 * self.steps

    @property
    def all_constant(self) -> bool:
        return all(layer.constant for layer in self.layers)


def refract(d, normal, n1, n2):
    """Snell refraction of the (possibly non-unit) direction ``d`` about ``normal``,
    normalised; returns (direction, total-internal-reflection flag)."""
    eta = n1 / n2
    cos_i = float(np.clip(np.dot(-np.asarray(d, dtype=np.float64), normal), -1.0, 1.0))
    sin2_t = eta**2 * (1.0 - cos_i**2)
    cos_t = math.sqrt(max(0.0, 1.0 - sin2_t))
    t = eta * np.asarray(d, dtype=np.float64) + (eta * cos_i - cos_t) * np.asarray(
        normal, dtype=np.float64
    )
    return t / np.linalg.norm(t), sin2_t > 1.0


def build_scene(cfg) -> SceneModel:
    """Derive the scene constants of ``cfg`` (a SimulationConfig, ours or the reference's)."""
    laser = cfg.laser
    theta = math.radians(laser.nadir_angle)
    phi = math.radians(laser.azimuth_angle)
    laser_dir = np.array(
        [math.sin(theta) * math.cos(phi), -math.cos(theta), math.sin(theta) * math.sin(phi)]
    )

    layers: List[LayerModel] = []
    depth_acc = 0.0
    for layer in cfg.water.layers:
        hg = getattr(layer, "henyey_greenstein_g", None)
        if hg is None:
            ff = layer.fournier_forand_parameters
            th, _, cdf = fournier_forand_table(ff.junge_slope, ff.refractive_index_ratio)
            bb = fournier_forand_backscatter(ff.junge_slope, ff.refractive_index_ratio)
        else:
            th, _, cdf = henyey_greenstein_table(float(hg))
            bb = henyey_greenstein_backscatter(float(hg))
        a0 = _value_at(layer.absorption_coefficient, 0.0, layer.height)
        b0 = _value_at(layer.scattering_coefficient, 0.0, layer.height)
        s0 = _value_at(layer.salinity, 0.0, layer.height)
        n0 = _value_at(layer.refractive_index, 0.0, layer.height)
        alpha = float(
            churnside_alpha(
                a0, b0, s0, laser.wavelength, cfg.scene.flying_height,
                laser.divergence_angle, bb,
            )
        )
        ssa = (alpha - a0) / alpha
        with np.errstate(divide="ignore", invalid="ignore"):
            slope = np.diff(th) / np.diff(cdf)
        weight, width32 = scatter_weight_table(th, cdf)
        top32 = float(np.float32(depth_acc))
        constant = _is_constant(layer)
        dla = dls = (0.0, 0.0, 0.0)
        if constant:
            dla, dls = adjoint_layer_terms(
                a0, b0, s0, laser.wavelength, cfg.scene.flying_height, laser.divergence_angle, bb,
                hg_g=None if hg is None else float(hg),
            )
        lut_z = lut_alpha = None
        if not constant:
            lut_z, lut_alpha = attenuation_lut(
                layer, laser.wavelength, cfg.scene.flying_height, laser.divergence_angle, bb
            )
        depth_acc = depth_acc + float(layer.height)
        layers.append(
            LayerModel(
                height=float(layer.height),
                bottom_depth=depth_acc,
                constant=_is_constant(layer),
                alpha64=alpha,
                alpha32=float(np.float32(alpha)),
                ssa32=float(np.float32(ssa)),
                speed32=float(np.float32(LIGHT_SPEED_AIR / n0)),
                n_top=float(n0),
                absorption=float(a0),
                ff_theta=th,
                ff_cdf=cdf,
                ff_slope=slope,
                backscatter=bb,
                scatter_weight=weight,
                bin_width32=float(width32),
                top32=top32,
                lut_z=lut_z,
                lut_alpha=lut_alpha,
                n_profile=_profile_code(layer.refractive_index),
                a_profile=_profile_code(layer.absorption_coefficient),
                dlog_alpha=dla,
                dlog_ssa=dls,
                hg_g=0.0 if hg is None else float(hg),
                dlog_weight_g=None if hg is None else hg_weight_dlog_g(float(hg), weight),
                dlog_sample_g=None if hg is None else hg_sample_dlog_g(float(hg)),
            )
        )
    depth = layers[-1].bottom_depth
    surface_y = -float(cfg.scene.flying_height)
    floor_y = -(float(cfg.scene.flying_height) + depth)

    sample_rate = cfg.sensor.sample_rate
    mult = cfg.sample_multiplier
    eff_rate = mult * sample_rate
    dt = 1 / eff_rate
    distance = floor_y / laser_dir[1]
    steps = int(1.5 * (distance * round(sample_rate)) / LIGHT_SPEED_AIR)

    n_water = layers[0].n_top
    f0 = ((1 - n_water) / (1 + n_water)) ** 2

    water_center = (surface_y / laser_dir[1]) * laser_dir
    refr, _ = refract(laser_dir, np.array([0.0, 1.0, 0.0]), 1.0, n_water)
    floor_center = water_center + (-depth / refr[1]) * refr

    hm = cfg.heatmap
    gate_start = gate_bins = 0
    gate = getattr(cfg, "waveform_gate", None)
    if gate is not None:
        # one waveform bin is one sample period (sample_multiplier integrator steps)
        gate_start = int(math.floor(float(gate[0]) * sample_rate))
        gate_bins = max(1, int(round(float(gate[1]) * sample_rate)))
        if gate_start + gate_bins > 2 * steps:
            raise ValueError("the waveform gate ends after the simulated time span")
    return SceneModel(
        sample_rate=int(sample_rate),
        sample_multiplier=int(mult),
        k=int(cfg.photon_mapping_k),
        dt=dt,
        steps=steps,
        total_substeps=steps * mult,
        surface_y=surface_y,
        floor_y=floor_y,
        depth=depth,
        laser_dir=laser_dir,
        laser_rot32=rotation_z_to(laser_dir),
        divergence=float(laser.divergence_angle),
        fov=float(cfg.sensor.field_of_view),
        aperture_radius=float(cfg.sensor.aperture_radius),
        pulse_sigma=float(laser.pulse_fwhm / (2 * np.sqrt(2 * np.log(2)))),
        effective_rate=float(eff_rate),
        n_water=n_water,
        f0=f0,
        seafloor_albedo=float(cfg.sea_floor.albedo),
        surface_albedo=float(cfg.sea_surface.albedo),
        roughness=float(cfg.sea_surface.roughness),
        flying_height=float(cfg.scene.flying_height),
        layers=layers,
        heatmap_enabled=bool(hm.enabled),
        gather_radius=(float(getattr(cfg, "gather_radius")) if getattr(cfg, "gather_radius", None) else None),
        heatmap_bins=int(hm.bins),
        heatmap_water_extent=float(hm.water_extent),
        heatmap_seafloor_extent=float(hm.seafloor_extent),
        water_center=water_center,
        floor_center=floor_center,
        gate_start=gate_start,
        gate_bins=gate_bins,
        slope_sigma=float(getattr(cfg.sea_surface, "slope_sigma", None) or 0.0),
    )
