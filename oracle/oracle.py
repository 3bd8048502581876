"""Python wrapper of the C oracle (alb_oracle.c).

TEST INFRASTRUCTURE ONLY: the parity checker of the GPU engine. Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module; nothing in
pyalbsim_gb300 does.

``oracle_run`` mirrors ``alb_sim.execution.linear.run_linear`` (execution/linear.py:77-117):
forward pass, photon maps in record order (build_photon_map_data.py:8-62), backward pass
with k-NN gathers, and returns the float64 waveform per channel.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIB_DIR, "liboracle.so")
SRC = os.path.join(HERE, "alb_oracle.c")


def build_oracle(force: bool = False) -> str:
    """Compile the oracle with gcc (no FMA contraction, so float rounding follows NumPy)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
        os.path.getmtime(SRC), os.path.getmtime(os.path.join(ROOT, "include", "albgpu.h"))
    ):
        return LIB
    os.makedirs(LIB_DIR, exist_ok=True)
    cmd = [
        "gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
        "-o", LIB + ".tmp", SRC, "-lm",
    ]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class _Rec(C.Structure):
    _fields_ = [
        ("channel", C.c_int32),
        ("photon", C.c_int32),
        ("step", C.c_int64),
        ("pos", C.c_double * 3),
        ("dir", C.c_double * 3),
        ("energy", C.c_float),
        ("time", C.c_float),
        ("fwi", C.c_float * 3),
        ("sfi", C.c_float * 3),
        ("score", C.c_float * 4),
    ]


_REC_DTYPE = np.dtype(
    [
        ("channel", np.int32),
        ("photon", np.int32),
        ("step", np.int64),
        ("pos", np.float64, 3),
        ("dir", np.float64, 3),
        ("energy", np.float32),
        ("time", np.float32),
        ("fwi", np.float32, 3),
        ("sfi", np.float32, 3),
        ("score", np.float32, 4),
    ],
    align=True,
)


class _Trace(C.Structure):
    _fields_ = [
        ("records", C.POINTER(_Rec)),
        ("n_records", C.c_int64),
        ("exit_pd", C.POINTER(C.c_double)),
        ("exit_f", C.POINTER(C.c_float)),
        ("hm_radius", C.POINTER(C.c_uint)),
    ]


_lib = None


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build_oracle())
        P = C.c_void_p
        lib.oracle_trace.argtypes = [P, C.c_int, C.c_uint64, C.c_uint64, C.c_uint64, P, P, P, C.POINTER(_Trace), C.c_int]
        lib.oracle_free.argtypes = [C.POINTER(_Trace)]
        lib.oracle_record_size.restype = C.c_int
        lib.oracle_knn.argtypes = [P, C.c_int64, P, C.c_int64, C.c_int, P, P, C.c_int]
        lib.oracle_set_knn_brute.argtypes = [C.c_int]
        lib.oracle_gather.argtypes = [
            P, C.c_int, P, P, P, P, P, P, C.c_int64, P, P, P, P, C.c_int64, P, P, P, P, P, P, P, C.c_int
        ]
        if lib.oracle_record_size() != _REC_DTYPE.itemsize:
            raise RuntimeError("oracle record layout mismatch")
        _lib = lib
    return _lib


def set_knn_brute(on: bool) -> None:
    """Neighbour searches of the oracle scan every map point (True, the checker of the
    tree) or descend its k-d tree (False, the default); both return the same neighbours."""
    _load().oracle_set_knn_brute(1 if on else 0)


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    """CPU restatement bound to one scene (a SceneModel from pyalbsim_gb300.scene)."""

    def __init__(self, scene, threads: int = 0):
        from pyalbsim_gb300._native import scene_struct  # struct packing only, no GPU call

        self.lib = _load()
        self.scene = scene
        self.params, self._keep = scene_struct(scene)
        self.threads = threads
        nb = scene.heatmap_bins
        self.hm_radius = np.zeros(nb * nb, np.uint32) if scene.heatmap_enabled else None

    def trace(self, forward: bool, n: int, seed: int = 0, first: int = 0, replay=None):
        """Returns (records structured array in (photon, step) order, exit-state dict)."""
        t = _Trace()
        t.hm_radius = (
            self.hm_radius.ctypes.data_as(C.POINTER(C.c_uint)) if (forward and self.hm_radius is not None) else None
        )
        offs = vals = taus = None
        if replay is not None:
            offs = np.ascontiguousarray(replay[0], np.int64)
            vals = np.ascontiguousarray(replay[1], np.float64)
            taus = np.ascontiguousarray(replay[2], np.float32)
        rc = self.lib.oracle_trace(
            C.byref(self.params), 0 if forward else 1, n, seed & 0xFFFFFFFFFFFFFFFF, first,
            _p(offs), _p(vals), _p(taus), C.byref(t), self.threads,
        )
        try:
            nrec = t.n_records
            buf = C.cast(t.records, C.POINTER(C.c_byte * (nrec * _REC_DTYPE.itemsize)))
            recs = np.frombuffer(bytes(buf.contents) if nrec else b"", dtype=_REC_DTYPE).copy()
            pd = np.ctypeslib.as_array(t.exit_pd, shape=(max(n, 1) * 6,))[: n * 6].reshape(n, 6).copy()
            f = np.ctypeslib.as_array(t.exit_f, shape=(max(n, 1) * 10,))[: n * 10].reshape(n, 10).copy()
        finally:
            self.lib.oracle_free(C.byref(t))
        if rc != 0:
            raise RuntimeError(f"oracle trace failed with code {rc}")
        exits = dict(
            pos=pd[:, :3], dir=pd[:, 3:], energy=f[:, 0], tau=f[:, 1], tau_target=f[:, 2], time=f[:, 3],
            fwi=f[:, 4:7], sfi=f[:, 7:10],
        )
        return recs, exits

    def knn(self, points, queries, k):
        pts = np.ascontiguousarray(points, np.float32)
        qs = np.ascontiguousarray(queries, np.float64)
        idx = np.empty((len(qs), k), np.int32)
        dist = np.empty((len(qs), k), np.float64)
        rc = self.lib.oracle_knn(_p(pts), len(pts), _p(qs), len(qs), k, _p(idx), _p(dist), self.threads)
        if rc != 0:
            raise IndexError("fewer map points than k")
        return dist, idx

    def gather(self, channel, m, q, waveform, heat_w=None, heat_f=None, jac=None):
        """m: dict pos/dir/energy/time/fwi/sfi (float32); q: dict pos/dir (float64), energy/time.
        jac (float64 [5, nbins], nullable) receives d waveform / d (a, b, g, albedo,
        roughness) from the "score" entries of m and q (float32 [n, 4])."""
        n = len(m["energy"])
        nq = len(q["energy"])
        rk = np.empty(nq, np.float64)
        arr = {k: np.ascontiguousarray(v, np.float32) for k, v in m.items()}
        qp = np.ascontiguousarray(q["pos"], np.float64)
        qd = np.ascontiguousarray(q["dir"], np.float64)
        qe = np.ascontiguousarray(q["energy"], np.float32)
        qt = np.ascontiguousarray(q["time"], np.float32)
        ms = qs = None
        if jac is not None:
            ms = np.ascontiguousarray(m["score"], np.float32)
            qs = np.ascontiguousarray(q["score"], np.float32)
        rc = self.lib.oracle_gather(
            C.byref(self.params), channel, _p(arr["pos"]), _p(arr["dir"]), _p(arr["energy"]), _p(arr["time"]),
            _p(arr.get("fwi")), _p(arr.get("sfi")), n, _p(qp), _p(qd), _p(qe), _p(qt), nq, _p(waveform), _p(rk),
            _p(heat_w), _p(heat_f), _p(ms), _p(qs), _p(jac), self.threads,
        )
        if rc == -2:
            raise IndexError(f"photon map of channel {channel} holds {n} records, fewer than k")
        if rc != 0:
            raise RuntimeError(f"oracle gather failed with code {rc}")
        return rk


def maps_from_records(recs, channels=4):
    """Per-channel dense float32 arrays in record order (build_photon_map_data)."""
    out = {}
    for c in range(channels):
        r = recs[recs["channel"] == c]
        out[c] = dict(
            pos=r["pos"].astype(np.float32),
            dir=r["dir"].astype(np.float32),
            energy=r["energy"].astype(np.float32),
            time=r["time"].astype(np.float32),
            fwi=r["fwi"].astype(np.float32),
            sfi=r["sfi"].astype(np.float32),
            score=r["score"].astype(np.float32),
            photon=r["photon"],
            step=r["step"],
        )
    return out


def queries_from_records(recs):
    out = {}
    for kind in range(3):
        r = recs[recs["channel"] == kind]
        out[kind] = dict(pos=r["pos"], dir=r["dir"], energy=r["energy"], time=r["time"], photon=r["photon"],
                         score=r["score"].astype(np.float32))
    return out


def oracle_run(scene, n_fwd, n_bwd, seed=0, replay_fwd=None, replay_bwd=None, threads=0, adjoint=False):
    """Forward + maps + backward + gathers; returns dict with waveforms (float64 [4, nbins])
    and, with adjoint=True, "jacobian" (float64 [5, 4, nbins]: d waveform / d (a, b, g,
    albedo, roughness))."""
    orc = Oracle(scene, threads=threads)
    frec, fexit = orc.trace(True, n_fwd, seed=seed, replay=replay_fwd)
    maps = maps_from_records(frec)
    brec, bexit = orc.trace(False, n_bwd, seed=seed, replay=replay_bwd)
    qs = queries_from_records(brec)
    nb = scene.n_bins
    wf = np.zeros((4, nb), np.float64)
    hb = scene.heatmap_bins * scene.heatmap_bins
    heat_w = np.zeros(hb, np.float64) if scene.heatmap_enabled else None
    heat_f = np.zeros(hb, np.float64) if scene.heatmap_enabled else None
    rks = {}
    jac = np.zeros((4, 5, nb), np.float64) if adjoint else None
    for ch, kind in ((0, 0), (1, 1), (2, 2), (3, 2)):
        if len(qs[kind]["energy"]) == 0:
            continue
        rks[ch] = orc.gather(ch, maps[ch], qs[kind], wf[ch], heat_w, heat_f,
                             jac=jac[ch] if adjoint else None)
    return dict(
        waveform=wf, maps=maps, queries=qs, fwd_exit=fexit, bwd_exit=bexit, rk=rks,
        heat_water=heat_w, heat_floor=heat_f, heat_radius=orc.hm_radius,
        jacobian=jac.transpose(1, 0, 2).copy() if adjoint else None,
    )


def kat_ggx(roughness, f0, wi, wo):
    lib = _load()
    lib.oracle_ggx_batch.argtypes = [C.c_double, C.c_double, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    wi = np.ascontiguousarray(wi, np.float64)
    wo = np.ascontiguousarray(wo, np.float64)
    out = np.empty(len(wi), np.float64)
    lib.oracle_ggx_batch(roughness, f0, _p(wi), len(wi), _p(wo), _p(out))
    return out


def kat_scatter_energy(scene, pdirs, view, layer=0):
    from pyalbsim_gb300._native import scene_struct

    lib = _load()
    lib.oracle_scatter_energy_batch.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    params, keep = scene_struct(scene)
    pd = np.ascontiguousarray(pdirs, np.float32)
    v = np.ascontiguousarray(view, np.float64)
    out = np.empty(len(pd), np.float64)
    lib.oracle_scatter_energy_batch(C.byref(params), layer, _p(pd), len(pd), _p(v), _p(out))
    return out


def abi_layout():
    lib = _load()
    out = np.zeros(7, np.int64)
    lib.oracle_abi_layout.argtypes = [C.c_void_p]
    lib.oracle_abi_layout(_p(out))
    return out
