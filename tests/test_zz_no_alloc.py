"""alb_knn_noalloc: the neighbour query for callers that cannot allocate device memory
(stream capture, real-time loops, frameworks that own the device pool). Called through the
C ABI with device buffers the test owns, twice in a row, and compared with the allocating
alb_knn on the same points and queries.

This file is named to be collected last, so a run that stops at its first failure has run
every other test before it; it also passes on its own in a fresh process."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _points(rng, m):
    core = rng.normal(scale=[0.3, 1.0, 0.3], size=(m // 2, 3)) + [0.0, -402.0, 0.0]
    halo = rng.uniform([-4.0, -406.0, -4.0], [4.0, -400.0, 4.0], size=(m - m // 2, 3))
    return np.concatenate([core, halo]).astype(np.float32)


def _queries(rng, pts, q):
    lo, hi = pts.min(0).astype(np.float64), pts.max(0).astype(np.float64)
    return rng.uniform(lo - 2.0, hi + 2.0, size=(q, 3))


def _noalloc(lib, torch, pts, qs, k):
    d_pts = torch.from_numpy(pts.reshape(-1)).cuda()
    d_q = torch.from_numpy(qs.reshape(-1)).cuda()
    d_idx = torch.empty(len(qs) * k, dtype=torch.int32, device="cuda")
    d_dist = torch.empty(len(qs) * k, dtype=torch.float64, device="cuda")
    rc = lib.alb_knn_noalloc(
        C.c_void_p(d_pts.data_ptr()), len(pts), C.c_void_p(d_q.data_ptr()), len(qs), k,
        C.c_void_p(d_idx.data_ptr()), C.c_void_p(d_dist.data_ptr()), None,
    )
    assert rc == 0, lib.alb_last_error(None).decode()
    torch.cuda.synchronize()
    return d_dist.cpu().numpy().reshape(-1, k), d_idx.cpu().numpy().reshape(-1, k)


def _assert_same_neighbours(d1, i1, d2, i2):
    # distances are computed by the same float64 expression on both paths: equal bits
    np.testing.assert_array_equal(d1, d2)
    for a, b, dd in zip(i1, i2, d1):
        strict = dd < dd[-1]  # sets agree except for exact ties at the k-th distance
        assert set(a[strict]) == set(b[strict])


def test_knn_noalloc_matches_allocating_knn_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fixtures import config_from_fixture, load
    from pyalbsim_gb300._native import load_library
    from pyalbsim_gb300.engine import GpuEngine

    lib = load_library()
    rng = np.random.default_rng(42)
    eng = GpuEngine(config_from_fixture(load("replay_small.npz")))
    try:
        for m, q, k in ((3000, 400, 100), (4096, 257, 32)):
            pts = _points(rng, m)
            qs = _queries(rng, pts, q)
            ref_d, ref_i = eng.ctx.knn(pts, qs, k)
            # two calls in a row on the shared static scratch
            d1, i1 = _noalloc(lib, torch, pts, qs, k)
            d2, i2 = _noalloc(lib, torch, pts, qs, k)
            _assert_same_neighbours(d1, i1, ref_d, ref_i)
            _assert_same_neighbours(d2, i2, ref_d, ref_i)
    finally:
        eng.close()


def test_knn_noalloc_matches_scipy_at_its_limits():
    """m = 4096 points and k = 256 (the entry point's maxima) against scipy's KDTree on the
    same float32 points: the same neighbour sets and float64 distances, two calls in a row."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from scipy.spatial import cKDTree

    from pyalbsim_gb300._native import load_library

    lib = load_library()
    rng = np.random.default_rng(4096)
    pts = _points(rng, 4096)
    qs = _queries(rng, pts, 300)
    ref_d, ref_i = cKDTree(pts.astype(np.float64)).query(qs, k=256)
    for _ in range(2):
        d, i = _noalloc(lib, torch, pts, qs, 256)
        np.testing.assert_allclose(d, ref_d, rtol=1e-12, atol=0.0)
        for a, b, dd in zip(i, ref_i, d):
            strict = dd < dd[-1]
            assert set(a[strict]) == set(b[strict])


def test_knn_noalloc_marks_a_query_without_an_answer():
    """A query with a NaN coordinate has no nearest neighbours: the call cannot report the
    device-side status synchronously, so all k slots of that query come back as index -1
    and distance NaN; the other queries of the same call are answered as usual."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from scipy.spatial import cKDTree

    from pyalbsim_gb300._native import load_library

    lib = load_library()
    rng = np.random.default_rng(11)
    pts = _points(rng, 1000)
    qs = _queries(rng, pts, 64)
    qs[5, 1] = np.nan
    k = 16
    d_pts = torch.from_numpy(pts.reshape(-1)).cuda()
    d_q = torch.from_numpy(qs.reshape(-1)).cuda()
    d_idx = torch.full((len(qs) * k,), 12345, dtype=torch.int32, device="cuda")
    d_dist = torch.zeros(len(qs) * k, dtype=torch.float64, device="cuda")
    rc = lib.alb_knn_noalloc(C.c_void_p(d_pts.data_ptr()), len(pts), C.c_void_p(d_q.data_ptr()), len(qs), k,
                             C.c_void_p(d_idx.data_ptr()), C.c_void_p(d_dist.data_ptr()), None)
    assert rc == 0  # asynchronous: the failure is in the output
    torch.cuda.synchronize()
    idx = d_idx.cpu().numpy().reshape(-1, k)
    dist = d_dist.cpu().numpy().reshape(-1, k)
    assert np.all(idx[5] == -1) and np.all(np.isnan(dist[5]))
    ok = np.arange(len(qs)) != 5
    ref_d, _ = cKDTree(pts.astype(np.float64)).query(qs[ok], k=k)
    assert np.all(idx[ok] >= 0)
    np.testing.assert_allclose(dist[ok], ref_d, rtol=1e-12, atol=0.0)


def test_knn_noalloc_rejects_oversize_input():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pyalbsim_gb300._native import load_library

    lib = load_library()
    d = torch.zeros(3 * 4097, dtype=torch.float32, device="cuda")
    q = torch.zeros(3, dtype=torch.float64, device="cuda")
    i = torch.zeros(8, dtype=torch.int32, device="cuda")
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = lib.alb_knn_noalloc(C.c_void_p(d.data_ptr()), 4097, C.c_void_p(q.data_ptr()), 1, 8,
                             C.c_void_p(i.data_ptr()), C.c_void_p(x.data_ptr()), None)
    assert rc == -1
    assert b"at most 4096 points" in lib.alb_last_error(None)
