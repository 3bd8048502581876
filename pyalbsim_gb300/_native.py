"""ctypes binding of libalbgpu.so (the C ABI declared in include/albgpu.h).

The library is the only compute path: importing this module on a machine without the
built library raises, and every call that returns a non-zero status raises the Python
exception the reference would raise for the same condition (ValueError for bad
configuration, IndexError for a photon map smaller than k, RuntimeError otherwise).
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from pyalbsim_gb300.build import LIB_PATH
from pyalbsim_gb300.scene import MAX_LAYERS, SceneModel

ALB_OK = 0
ALB_ERR_INVALID = -1
ALB_ERR_TOO_FEW = -2
ALB_ERR_CAPACITY = -3
ALB_ERR_CUDA = -4
ALB_ERR_ITER_CAP = -5
ALB_ERR_REPLAY = -6
ALB_ERR_STATE = -7

ALB_FORWARD, ALB_BACKWARD = 0, 1
ALB_OPT_KEEP_EXIT_STATES = 1
ALB_OPT_KEEP_RECORD_IDS = 2
ALB_OPT_PRECISE = 3
ALB_OPT_MAP_CAPACITY = 4
ALB_OPT_SORT_QUERIES = 5
ALB_OPT_STREAM = 6
ALB_OPT_ADJOINT = 7
ALB_ADJ_PARAMS = 6  # depth, a, b, g, albedo, roughness

PHASE_DIVISIONS = 18000


class AlbLayer(C.Structure):
    _fields_ = [
        ("bottom_depth", C.c_double),
        ("speed", C.c_double),
        ("alpha", C.c_float),
        ("ssa", C.c_float),
        ("absorption", C.c_double),
        ("bin_width", C.c_double),
        ("phase_theta", C.POINTER(C.c_double)),
        ("phase_cdf", C.POINTER(C.c_double)),
        ("phase_slope", C.POINTER(C.c_double)),
        ("scatter_weight", C.POINTER(C.c_double)),
        ("profiled", C.c_int32),
        ("lut_n", C.c_int32),
        ("lut_z", C.POINTER(C.c_float)),
        ("lut_alpha", C.POINTER(C.c_double)),
        ("n_kind", C.c_int32),
        ("a_kind", C.c_int32),
        ("n_start", C.c_double),
        ("n_end", C.c_double),
        ("a_start", C.c_double),
        ("a_end", C.c_double),
        ("height", C.c_double),
        ("top32", C.c_double),
        ("dlog_alpha", C.c_double * 3),
        ("dlog_ssa", C.c_double * 3),
        ("hg_g", C.c_double),
        ("dlog_weight_g", C.POINTER(C.c_double)),
        ("dlog_sample_g", C.POINTER(C.c_double)),
    ]


class AlbSceneParams(C.Structure):
    _fields_ = [
        ("dt", C.c_double),
        ("steps", C.c_int64),
        ("sample_multiplier", C.c_int32),
        ("k", C.c_int32),
        ("surface_y", C.c_double),
        ("floor_y", C.c_double),
        ("speed_air", C.c_double),
        ("n_water", C.c_double),
        ("f0", C.c_double),
        ("seafloor_albedo", C.c_double),
        ("surface_albedo", C.c_double),
        ("roughness", C.c_double),
        ("laser_dir", C.c_double * 3),
        ("laser_rot", C.c_float * 9),
        ("divergence", C.c_double),
        ("fov", C.c_double),
        ("aperture_radius", C.c_double),
        ("pulse_sigma", C.c_double),
        ("effective_rate", C.c_double),
        ("n_layers", C.c_int32),
        ("heatmap_enabled", C.c_int32),
        ("heatmap_bins", C.c_int32),
        ("reserved0", C.c_int32),
        ("heatmap_water_extent", C.c_double),
        ("heatmap_floor_extent", C.c_double),
        ("water_center", C.c_double * 3),
        ("floor_center", C.c_double * 3),
        ("layers", AlbLayer * MAX_LAYERS),
        ("gather_radius", C.c_double),
        ("gate_start", C.c_int64),
        ("gate_bins", C.c_int64),
        ("slope_sigma", C.c_double),
    ]


class AlbReplay(C.Structure):
    _fields_ = [
        ("offsets", C.POINTER(C.c_int64)),
        ("values", C.POINTER(C.c_double)),
        ("tau", C.POINTER(C.c_float)),
        ("n_values", C.c_uint64),
    ]


class AlbBatchInstance(C.Structure):
    _fields_ = [
        ("scene", C.POINTER(AlbSceneParams)),
        ("n_forward", C.c_uint64),
        ("n_backward", C.c_uint64),
        ("seed", C.c_uint64),
        ("waveform", C.POINTER(C.c_double)),
        ("jacobian", C.POINTER(C.c_double)),
        ("status", C.c_int32),
        ("device_ms", C.c_float),
    ]


class AlbBatchOptions(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("streams", C.c_int32),
        ("precise", C.c_int32),
        ("adjoint", C.c_int32),
    ]


EXPORTED = [
    "alb_adjoint",
    "alb_batch_run",
    "alb_export_map_scores",
    "alb_get_jacobian",
    "alb_create",
    "alb_destroy",
    "alb_last_error",
    "alb_set_option",
    "alb_trace",
    "alb_build_maps",
    "alb_map_size",
    "alb_export_map",
    "alb_get_heatmaps",
    "alb_get_waveform",
    "alb_get_waveform_f64",
    "alb_reset_waveform",
    "alb_export_exit_states",
    "alb_query_count",
    "alb_export_queries",
    "alb_knn",
    "alb_stats",
    "alb_phase_times",
    "alb_reset",
    "alb_knn_noalloc",
]

PHASES = ["trace_fwd", "map_build", "trace_bwd", "query_sort", "gather_bottom", "gather_scatter",
          "gather_surface_reflection", "gather_transmission_up"]

_P = C.c_void_p
_lib = None


def load_library(path: str = LIB_PATH):
    """Load libalbgpu.so and declare its prototypes; raises if it was never built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -m pyalbsim_gb300.build` "
            "(there is no CPU fallback)"
        )
    lib = C.CDLL(path)
    lib.alb_create.argtypes = [C.POINTER(AlbSceneParams), C.c_int, C.POINTER(_P)]
    lib.alb_destroy.argtypes = [_P]
    lib.alb_destroy.restype = None
    lib.alb_last_error.argtypes = [_P]
    lib.alb_last_error.restype = C.c_char_p
    lib.alb_set_option.argtypes = [_P, C.c_int, C.c_int64]
    lib.alb_trace.argtypes = [_P, C.c_int, C.c_uint64, C.c_uint64, C.c_uint64, C.POINTER(AlbReplay)]
    lib.alb_build_maps.argtypes = [_P]
    lib.alb_map_size.argtypes = [_P, C.c_int, C.POINTER(C.c_uint64)]
    lib.alb_export_map.argtypes = [_P, C.c_int, _P, _P, _P, _P, _P, _P, _P, C.c_size_t]
    lib.alb_get_heatmaps.argtypes = [_P, _P, _P, _P, C.c_size_t]
    lib.alb_get_waveform.argtypes = [_P, C.c_int, _P, C.c_size_t]
    lib.alb_get_waveform_f64.argtypes = [_P, C.c_int, _P, C.c_size_t]
    lib.alb_reset_waveform.argtypes = [_P]
    lib.alb_export_exit_states.argtypes = [_P, _P, _P, _P, _P, _P, _P, _P, _P, C.c_size_t]
    lib.alb_query_count.argtypes = [_P, C.c_int, C.POINTER(C.c_uint64)]
    lib.alb_export_queries.argtypes = [_P, C.c_int, _P, _P, _P, _P, _P, _P, _P, C.c_size_t]
    lib.alb_knn.argtypes = [_P, _P, C.c_uint64, _P, C.c_uint64, C.c_int, _P, _P]
    lib.alb_stats.argtypes = [_P, _P, C.c_int]
    lib.alb_phase_times.argtypes = [_P, _P, _P, _P, C.c_int]
    lib.alb_reset.argtypes = [_P]
    lib.alb_knn_noalloc.argtypes = [_P, C.c_uint64, _P, C.c_uint64, C.c_int, _P, _P, _P]
    lib.alb_get_jacobian.argtypes = [_P, C.c_int, C.c_int, _P, C.c_size_t]
    lib.alb_adjoint.argtypes = [_P, _P, C.c_size_t, _P]
    lib.alb_export_map_scores.argtypes = [_P, C.c_int, _P, C.c_size_t]
    lib.alb_batch_run.argtypes = [C.POINTER(AlbBatchInstance), C.c_uint64, C.POINTER(AlbBatchOptions)]
    _lib = lib
    return lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def raise_for(code: int, message: str):
    if code == ALB_OK:
        return
    if code == ALB_ERR_INVALID:
        raise ValueError(message)
    if code == ALB_ERR_TOO_FEW:
        raise IndexError(message)
    raise RuntimeError(f"albgpu error {code}: {message}")


def scene_struct(scene: SceneModel):
    """Pack a SceneModel into AlbSceneParams; returns (struct, keepalive arrays)."""
    p = AlbSceneParams()
    keep = []
    p.dt = scene.dt
    p.steps = scene.steps
    p.sample_multiplier = scene.sample_multiplier
    p.k = scene.k
    p.surface_y = scene.surface_y
    p.floor_y = scene.floor_y
    p.speed_air = float(np.float32(2.998e8))
    p.n_water = scene.n_water
    p.f0 = scene.f0
    p.seafloor_albedo = scene.seafloor_albedo
    p.surface_albedo = scene.surface_albedo
    p.roughness = scene.roughness
    for i in range(3):
        p.laser_dir[i] = float(scene.laser_dir[i])
        p.water_center[i] = float(scene.water_center[i])
        p.floor_center[i] = float(scene.floor_center[i])
    rot = np.asarray(scene.laser_rot32, dtype=np.float32).reshape(-1)
    for i in range(9):
        p.laser_rot[i] = float(rot[i])
    p.divergence = scene.divergence
    p.fov = scene.fov
    p.aperture_radius = scene.aperture_radius
    p.pulse_sigma = scene.pulse_sigma
    p.effective_rate = scene.effective_rate
    if len(scene.layers) > MAX_LAYERS:
        raise ValueError(f"at most {MAX_LAYERS} water layers are supported")
    p.n_layers = len(scene.layers)
    p.gather_radius = float(scene.gather_radius or 0.0)
    p.gate_start = int(scene.gate_start)
    p.gate_bins = int(scene.gate_bins)
    p.slope_sigma = float(scene.slope_sigma)
    p.heatmap_enabled = int(scene.heatmap_enabled)
    p.heatmap_bins = scene.heatmap_bins
    p.heatmap_water_extent = scene.heatmap_water_extent
    p.heatmap_floor_extent = scene.heatmap_seafloor_extent
    for i, layer in enumerate(scene.layers):
        L = p.layers[i]
        L.bottom_depth = layer.bottom_depth
        L.speed = layer.speed32
        L.alpha = layer.alpha32
        L.ssa = layer.ssa32
        L.absorption = layer.absorption
        L.bin_width = layer.bin_width32
        th = np.ascontiguousarray(layer.ff_theta, dtype=np.float64)
        cdf = np.ascontiguousarray(layer.ff_cdf, dtype=np.float64)
        sl = np.zeros(PHASE_DIVISIONS, dtype=np.float64)
        sl[: PHASE_DIVISIONS - 1] = layer.ff_slope
        w = np.ascontiguousarray(layer.scatter_weight, dtype=np.float64)
        keep += [th, cdf, sl, w]
        L.phase_theta = th.ctypes.data_as(C.POINTER(C.c_double))
        L.phase_cdf = cdf.ctypes.data_as(C.POINTER(C.c_double))
        L.phase_slope = sl.ctypes.data_as(C.POINTER(C.c_double))
        L.scatter_weight = w.ctypes.data_as(C.POINTER(C.c_double))
        L.height = layer.height
        L.top32 = layer.top32
        L.profiled = int(not layer.constant)
        if not layer.constant:
            lz = np.ascontiguousarray(layer.lut_z, dtype=np.float32)
            la = np.ascontiguousarray(layer.lut_alpha, dtype=np.float64)
            keep += [lz, la]
            L.lut_n = len(lz)
            L.lut_z = lz.ctypes.data_as(C.POINTER(C.c_float))
            L.lut_alpha = la.ctypes.data_as(C.POINTER(C.c_double))
            L.n_kind, L.n_start, L.n_end = layer.n_profile
            L.a_kind, L.a_start, L.a_end = layer.a_profile
        for j in range(3):
            L.dlog_alpha[j] = float(layer.dlog_alpha[j])
            L.dlog_ssa[j] = float(layer.dlog_ssa[j])
        L.hg_g = float(layer.hg_g)
        if layer.dlog_weight_g is not None:
            dw = np.ascontiguousarray(layer.dlog_weight_g, dtype=np.float64)
            keep.append(dw)
            L.dlog_weight_g = dw.ctypes.data_as(C.POINTER(C.c_double))
        if getattr(layer, "dlog_sample_g", None) is not None:
            ds = np.ascontiguousarray(layer.dlog_sample_g, dtype=np.float64)
            keep.append(ds)
            L.dlog_sample_g = ds.ctypes.data_as(C.POINTER(C.c_double))
    return p, keep


class NativeContext:
    """Owner of one AlbCtx; thin methods over the C ABI with NumPy buffers."""

    def __init__(self, scene: SceneModel, device: int = 0):
        self.lib = load_library()
        self.scene = scene
        self._params, self._keep = scene_struct(scene)
        h = C.c_void_p()
        rc = self.lib.alb_create(C.byref(self._params), device, C.byref(h))
        if rc != ALB_OK:
            raise_for(rc, self.lib.alb_last_error(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.alb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != ALB_OK:
            raise_for(rc, self.lib.alb_last_error(self.h).decode())

    def set_option(self, key: int, value: int):
        self._check(self.lib.alb_set_option(self.h, key, int(value)))

    def trace(self, forward: bool, n: int, seed: int = 0, first: int = 0, replay=None):
        rp = None
        if replay is not None:
            offsets, values, tau = replay
            offsets = np.ascontiguousarray(offsets, dtype=np.int64)
            values = np.ascontiguousarray(values, dtype=np.float64)
            tau = np.ascontiguousarray(tau, dtype=np.float32)
            if len(offsets) != n + 1:
                raise ValueError("replay offsets must have n + 1 entries")
            rp = AlbReplay(
                offsets.ctypes.data_as(C.POINTER(C.c_int64)),
                values.ctypes.data_as(C.POINTER(C.c_double)),
                tau.ctypes.data_as(C.POINTER(C.c_float)),
                len(values),
            )
            self._replay_keep = (offsets, values, tau)
        pass_ = ALB_FORWARD if forward else ALB_BACKWARD
        self._check(
            self.lib.alb_trace(
                self.h, pass_, n, seed & 0xFFFFFFFFFFFFFFFF, first, C.byref(rp) if rp is not None else None
            )
        )

    def build_maps(self):
        self._check(self.lib.alb_build_maps(self.h))

    def map_size(self, channel: int) -> int:
        out = C.c_uint64()
        self._check(self.lib.alb_map_size(self.h, channel, C.byref(out)))
        return out.value

    def export_map(self, channel: int):
        """(pos, dir, energy, time, fwi, sfi, photon_id) of one channel's records."""
        n = self.map_size(channel)
        pos = np.empty((n, 3), np.float32)
        d = np.empty((n, 3), np.float32)
        e = np.empty(n, np.float32)
        t = np.empty(n, np.float32)
        fwi = np.empty((n, 3), np.float32)
        sfi = np.empty((n, 3), np.float32)
        pid = np.empty(n, np.int64)
        self._check(
            self.lib.alb_export_map(
                self.h, channel, _ptr(pos), _ptr(d), _ptr(e), _ptr(t), _ptr(fwi), _ptr(sfi), _ptr(pid), n
            )
        )
        return pos, d, e, t, fwi, sfi, pid

    def heatmaps(self):
        b2 = self.scene.heatmap_bins * self.scene.heatmap_bins
        w = np.empty(b2, np.float64)
        f = np.empty(b2, np.float64)
        r = np.empty(b2, np.float32)
        self._check(self.lib.alb_get_heatmaps(self.h, _ptr(w), _ptr(f), _ptr(r), b2))
        return w, f, r

    def waveform(self, channel: int, f64: bool = False) -> np.ndarray:
        nb = self.scene.n_bins
        if f64:
            out = np.empty(nb, np.float64)
            self._check(self.lib.alb_get_waveform_f64(self.h, channel, _ptr(out), nb))
        else:
            out = np.empty(nb, np.float32)
            self._check(self.lib.alb_get_waveform(self.h, channel, _ptr(out), nb))
        return out

    def reset_waveform(self):
        self._check(self.lib.alb_reset_waveform(self.h))

    def exit_states(self, n: int):
        pos = np.empty((n, 3), np.float64)
        d = np.empty((n, 3), np.float64)
        f = {k: np.empty(n, np.float32) for k in ("energy", "tau", "tau_target", "time")}
        fwi = np.empty((n, 3), np.float32)
        sfi = np.empty((n, 3), np.float32)
        self._check(
            self.lib.alb_export_exit_states(
                self.h, _ptr(pos), _ptr(d), _ptr(f["energy"]), _ptr(f["tau"]), _ptr(f["tau_target"]),
                _ptr(f["time"]), _ptr(fwi), _ptr(sfi), n,
            )
        )
        return dict(pos=pos, dir=d, fwi=fwi, sfi=sfi, **f)

    def query_count(self, kind: int) -> int:
        out = C.c_uint64()
        self._check(self.lib.alb_query_count(self.h, kind, C.byref(out)))
        return out.value

    def export_queries(self, kind: int):
        n = self.query_count(kind)
        pos = np.empty((n, 3), np.float64)
        d = np.empty((n, 3), np.float32)
        e = np.empty(n, np.float32)
        t = np.empty(n, np.float32)
        pid = np.empty(n, np.int64)
        rk = np.empty(n, np.float64)
        rk2 = np.empty(n, np.float64)
        self._check(
            self.lib.alb_export_queries(
                self.h, kind, _ptr(pos), _ptr(d), _ptr(e), _ptr(t), _ptr(pid), _ptr(rk), _ptr(rk2), n
            )
        )
        return dict(pos=pos, dir=d, energy=e, time=t, id=pid, rk=rk, rk2=rk2)

    def jacobian(self) -> np.ndarray:
        """d waveform / d (a, b, g, albedo, roughness): float64 [5, channels, nbins]."""
        nb = self.scene.n_bins
        out = np.zeros((ALB_ADJ_PARAMS - 1, 4, nb), np.float64)
        for p in range(1, ALB_ADJ_PARAMS):
            for c in range(4):
                self._check(self.lib.alb_get_jacobian(self.h, p, c, _ptr(out[p - 1, c]), nb))
        return out

    def adjoint(self, dL_dw: np.ndarray) -> np.ndarray:
        """grad[1:] = sum dL_dw * J for (a, b, g, albedo, roughness); grad[0] (depth) is NaN."""
        d = np.ascontiguousarray(dL_dw, np.float64)
        if d.shape != (4, self.scene.n_bins):
            raise ValueError("dL_dw must have shape (channels, nbins)")
        g = np.empty(ALB_ADJ_PARAMS, np.float64)
        self._check(self.lib.alb_adjoint(self.h, _ptr(d), self.scene.n_bins, _ptr(g)))
        return g

    def export_map_scores(self, channel: int) -> np.ndarray:
        n = self.map_size(channel)
        out = np.empty((n, 4), np.float32)
        self._check(self.lib.alb_export_map_scores(self.h, channel, _ptr(out), n))
        return out

    def knn(self, points: np.ndarray, queries: np.ndarray, k: int):
        pts = np.ascontiguousarray(points, dtype=np.float32)
        qs = np.ascontiguousarray(queries, dtype=np.float64)
        idx = np.empty((len(qs), k), np.int32)
        dist = np.empty((len(qs), k), np.float64)
        self._check(self.lib.alb_knn(self.h, _ptr(pts), len(pts), _ptr(qs), len(qs), k, _ptr(idx), _ptr(dist)))
        return dist, idx

    def stats(self):
        """Counters of the last trace (events, photons), of the last forward trace
        (forward_events, forward_photons) and of the gathers (per channel: leaves
        opened, internal nodes expanded, candidate reductions, queries, and queries whose
        answer a buffer bound made inexact, which takes mass ties of distances)."""
        out = np.zeros(32, np.int64)
        self._check(self.lib.alb_stats(self.h, _ptr(out), 32))
        st = {"events": int(out[0]), "photons": int(out[1]), "launches": int(out[2]),
              "forward_events": int(out[28]), "forward_photons": int(out[29]),
              "search_retries": int(out[30])}
        for c, name in enumerate(("bottom", "scatter", "surface_reflection", "transmission_up")):
            lv, nd, se, nq = (int(x) for x in out[4 + 4 * c: 8 + 4 * c])
            st[f"gather_{name}"] = {
                "queries": nq,
                "leaves_per_query": lv / nq if nq else 0.0,
                "nodes_per_query": nd / nq if nq else 0.0,
                "selects_per_query": se / nq if nq else 0.0,
                "inexact": int(out[24 + c]),
            }
        return st

    def phase_times(self, reset: bool = False):
        ms = np.zeros(len(PHASES), np.float64)
        calls = np.zeros(len(PHASES), np.int64)
        gathers = np.zeros(4, np.int64)
        self._check(self.lib.alb_phase_times(self.h, _ptr(ms), _ptr(calls), _ptr(gathers), int(reset)))
        return {p: (float(m), int(c)) for p, m, c in zip(PHASES, ms, calls)}, gathers

    def reset(self):
        self._check(self.lib.alb_reset(self.h))


def batch_run(scenes, n_forward, n_backward, seeds, streams=4, precise=False, adjoint=False, device=0,
              jacobian_mask=None):
    """alb_batch_run over SceneModels: returns (waveforms: list of float64 [4, nbins],
    jacobians: list of float64 [5, 4, nbins] (None for masked-out instances) or None,
    statuses int32 [n], device_ms [n]). With adjoint, ``jacobian_mask`` (bools) selects the
    instances that accumulate a Jacobian; the others run plain. Instances that failed keep a
    zero waveform and a non-zero status."""
    lib = load_library()
    n = len(scenes)
    structs, keep, waves, jacs = [], [], [], []
    arr = (AlbBatchInstance * max(n, 1))()
    for i, sc in enumerate(scenes):
        p, k = scene_struct(sc)
        structs.append(p)
        keep.append(k)
        w = np.zeros((4, sc.n_bins), np.float64)
        want = adjoint and (jacobian_mask is None or bool(jacobian_mask[i]))
        j = np.zeros((5, 4, sc.n_bins), np.float64) if want else None
        waves.append(w)
        jacs.append(j)
        arr[i].scene = C.pointer(p)
        arr[i].n_forward = int(n_forward[i])
        arr[i].n_backward = int(n_backward[i])
        arr[i].seed = int(seeds[i]) & 0xFFFFFFFFFFFFFFFF
        arr[i].waveform = w.ctypes.data_as(C.POINTER(C.c_double))
        arr[i].jacobian = j.ctypes.data_as(C.POINTER(C.c_double)) if want else None
    opt = AlbBatchOptions(device, int(streams), int(bool(precise)), int(bool(adjoint)))
    rc = lib.alb_batch_run(arr, n, C.byref(opt))
    raise_for(rc, lib.alb_last_error(None).decode())
    status = np.array([arr[i].status for i in range(n)], np.int32)
    ms = np.array([arr[i].device_ms for i in range(n)], np.float64)
    return waves, (jacs if adjoint else None), status, ms
