"""The local phase of the ridge MST on the GPU (m16_ridge_mst_local, Boruvka
rounds in the (weight, i, j) order) against SciPy's Kruskal in the same order
(ridge_mst.py, local="host") and against the dense stable Kruskal of the
oracle (oracle/adjust.py:stable_mst, the reference's
minimum_spanning_tree(squareform(pdist(...))) with equal distances in (i, j)
order): the same edge sets on point sets full of equal distances, isotropic
and anisotropic voxel sizes; the adjuster's ridge directions and cleaning
with the GPU tree equal the reference logic."""
import contextlib
import ctypes
import io

import numpy as np
import pytest

from oracle import adjust as A

pytestmark = pytest.mark.gpu


def _set(a, b):
    return set(zip(np.minimum(a, b).tolist(), np.maximum(a, b).tolist()))


def _clouds(rng, n_clusters, size, spread):
    """Clusters of integer points (many equal distances), shuffled."""
    pts = np.unique(np.concatenate([rng.randint(0, size, (60, 3)) + rng.randint(0, spread, 3)
                                    for _ in range(n_clusters)]), axis=0)
    return pts[rng.permutation(len(pts))]


@pytest.mark.parametrize("vs", [(1, 1, 1), (1.5, 0.7, 1.2), (1, 1, 3), (0.5, 0.5, 0.5)])
def test_local_phase_equals_host_kruskal(vs):
    from miccai2016_gb300 import ridge_mst as M
    rng = np.random.RandomState(int(sum(vs) * 10))
    vsa = np.asarray(vs, np.float64)
    r, offsets = M._local_offsets(vsa)
    for k in range(4):
        pts = _clouds(rng, 6 + 3 * k, 8, 40)
        g = M._local_mst_gpu(pts.astype(np.int64), vsa, r, offsets)
        h = M._local_mst_host(pts.astype(np.int64), vsa, r, offsets)
        assert _set(*g) == _set(*h)
        assert len(g[0]) == len(h[0])


def test_dense_ridge_band_equals_host_kruskal():
    from miccai2016_gb300 import ridge_mst as M
    rng = np.random.RandomState(7)
    t = np.linspace(0, 8 * np.pi, 30000)
    band = np.stack([t * 10, 60 + 40 * np.sin(t), 60 + 40 * np.cos(t)], -1)
    pts = np.unique(np.round(band[:, None, :] + rng.randint(-2, 3, (len(t), 6, 3))).reshape(-1, 3), axis=0)
    pts = pts[pts.min(1) >= 0].astype(np.int64)
    for vs in [(1, 1, 1), (0.8, 1.1, 1.0)]:
        vsa = np.asarray(vs, np.float64)
        r, offsets = M._local_offsets(vsa)
        assert _set(*M._local_mst_gpu(pts, vsa, r, offsets)) == _set(*M._local_mst_host(pts, vsa, r, offsets))


@pytest.mark.parametrize("vs", [(1, 1, 1), (1.5, 0.7, 1.2)])
def test_whole_tree_equals_the_dense_stable_kruskal(vs):
    from miccai2016_gb300.ridge_mst import ridge_mst_edges
    rng = np.random.RandomState(int(sum(vs) * 7))
    for _ in range(3):
        pts = np.unique(np.concatenate([rng.randint(0, 10, (120, 3)) + rng.randint(0, 35, 3) for _ in range(4)]),
                        axis=0)
        pts = pts[rng.permutation(len(pts))]
        a, b = ridge_mst_edges(pts, vs, local="gpu")
        t = A.stable_mst(pts, vs).tocoo()
        assert _set(a, b) == _set(t.row, t.col)


def test_adjuster_with_the_gpu_tree_matches_the_reference_logic():
    from miccai2016_gb300.adjust_directions import AdvancedAdjuster
    rng = np.random.RandomState(4)
    shape = (24, 24, 24)
    ridge = np.zeros(shape, np.float32)
    for _ in range(6):
        p = rng.randint(2, 22, 3)
        for _ in range(rng.randint(1, 25)):
            ridge[tuple(np.clip(p, 0, 23))] = 1
            p = p + rng.randint(-1, 2, 3)
    main = rng.normal(size=shape + (3,)).astype(np.float32)
    obj = AdvancedAdjuster((0.01, 0.3), np.zeros(shape + (3,), np.float32), np.zeros(shape, np.float32))
    assert obj.mst_local == "gpu"
    c1, d1 = A.adjust_ridge_directions(ridge, main, (1.0, 1.0, 1.0))
    c2, d2 = obj._adjust_ridge_directions(ridge, main)
    assert np.array_equal(c1, c2)
    assert np.array_equal(np.ascontiguousarray(d1).view(np.uint32), np.ascontiguousarray(d2).view(np.uint32))
    with contextlib.redirect_stdout(io.StringIO()):
        k1 = A.clean_ridge(ridge, c1, d1, (1.0, 1.0, 1.0))
        k2 = obj._do_clean_ridge(ridge, c2, d2)
    assert np.array_equal(k1, k2)


def test_duplicate_or_outside_points_are_rejected():
    import torch
    from miccai2016_gb300 import _native as N
    L = N.lib()
    vs = (ctypes.c_double * 3)(1, 1, 1)
    offs = np.array([[0, 0, 1], [0, 1, 0], [1, 0, 0]], np.int32)

    def call(pts, lo, dims):
        d = torch.from_numpy(np.ascontiguousarray(pts, np.int32)).cuda()
        lo = np.asarray(lo, np.int32)
        dims = np.asarray(dims, np.int32)
        e = torch.empty((len(pts), 2), dtype=torch.int32, device="cuda")
        ws = N.workspace(L.m16_ridge_mst_workspace_bytes(len(pts), dims.ctypes.data_as(ctypes.c_void_p), 3))
        n = ctypes.c_int64(0)
        return L.m16_ridge_mst_local(N.ptr(d), len(pts), lo.ctypes.data_as(ctypes.c_void_p),
                                     dims.ctypes.data_as(ctypes.c_void_p), vs, offs.ctypes.data_as(ctypes.c_void_p),
                                     3, 1.7320508075688772, N.ptr(e), ctypes.byref(n), N.ptr(ws), ws.numel(),
                                     N.stream_ptr()), n.value
    ok = call([[0, 0, 0], [0, 0, 1], [0, 1, 1]], (0, 0, 0), (1, 2, 2))
    assert ok == (N.M16_OK, 2)
    assert call([[0, 0, 0], [0, 0, 1], [0, 0, 1]], (0, 0, 0), (1, 1, 2))[0] == N.M16_ERR_BAD_ARG
    assert call([[0, 0, 0], [0, 0, 5]], (0, 0, 0), (1, 1, 2))[0] == N.M16_ERR_BAD_ARG


def _segments(rng, n_seg, big):
    """A ridge-like point set: one long thick curve and many short specks,
    far apart, with equal distances everywhere (integer points)."""
    t = np.linspace(0, 6 * np.pi, big)
    curve = np.stack([t * 6, 80 + 50 * np.sin(t), 80 + 50 * np.cos(t)], -1)
    pts = [np.round(curve[:, None, :] + rng.randint(-1, 2, (big, 3, 3))).reshape(-1, 3)]
    for _ in range(n_seg):
        c = rng.randint(5, 150, 3)
        pts.append(c + np.cumsum(rng.randint(-1, 2, (rng.randint(1, 40), 3)), axis=0))
    pts = np.unique(np.concatenate(pts), axis=0)
    pts = pts[pts.min(1) >= 0].astype(np.int64)
    return pts[rng.permutation(len(pts))]


@pytest.mark.parametrize("seed", range(4))
def test_device_joins_equal_the_host_joins(seed):
    """m16_ridge_forest_joins (the global phase on the device) gives the edge
    set of the k-d tree joins on the host, and of the oracle's stable Kruskal
    where that fits."""
    from miccai2016_gb300.ridge_mst import ridge_mst_edges
    rng = np.random.RandomState(30 + seed)
    pts = _segments(rng, 10 + 10 * seed, 600 + 400 * seed)
    a, b = ridge_mst_edges(pts, (1, 1, 1), local="gpu")
    h = ridge_mst_edges(pts, (1, 1, 1), local="gpu", joins_on_device=False)
    assert len(a) == len(pts) - 1
    assert _set(a, b) == _set(*h)
    if seed == 0:
        t = A.prim_mst(pts, (1, 1, 1)).tocoo()
        assert _set(a, b) == _set(t.row, t.col)


def test_device_joins_on_clusters_full_of_ties():
    from miccai2016_gb300.ridge_mst import ridge_mst_edges
    rng = np.random.RandomState(5)
    for _ in range(3):
        pts = np.unique(np.concatenate([rng.randint(0, 6, (40, 3)) * 3 + rng.randint(0, 60, 3)
                                        for _ in range(12)]), axis=0)
        pts = pts[rng.permutation(len(pts))].astype(np.int64)
        a, b = ridge_mst_edges(pts, (1, 1, 1), local="gpu")
        t = A.stable_mst(pts, (1, 1, 1)).tocoo()
        assert _set(a, b) == _set(t.row, t.col)


def test_device_joins_reject_and_decline():
    import torch
    from miccai2016_gb300 import _native as N
    L = N.lib()
    pts = torch.tensor([[0, 0, 0], [0, 0, 9], [40000, 0, 0]], dtype=torch.int32, device="cuda")
    e = torch.zeros((0, 2), dtype=torch.int32, device="cuda")
    ja, jb = np.zeros(2, np.int32), np.zeros(2, np.int32)
    nj = ctypes.c_int64(0)
    ws = N.workspace(L.m16_ridge_forest_joins_workspace_bytes(3))
    vp = lambda x: x.ctypes.data_as(ctypes.c_void_p)
    ea, eb = e[:, 0].contiguous(), e[:, 1].contiguous()
    # a coordinate beyond 32767: rejected
    assert L.m16_ridge_forest_joins(N.ptr(pts), 3, N.ptr(ea), N.ptr(eb), 0, 10 ** 9, vp(ja), vp(jb),
                                    ctypes.byref(nj), N.ptr(ws), ws.numel(), N.stream_ptr()) == N.M16_ERR_BAD_ARG
    pts[2, 0] = 7
    # a budget too small for the search: declined, nothing written
    assert L.m16_ridge_forest_joins(N.ptr(pts), 3, N.ptr(ea), N.ptr(eb), 0, 1, vp(ja), vp(jb),
                                    ctypes.byref(nj), N.ptr(ws), ws.numel(), N.stream_ptr()) == N.M16_ERR_TOO_LARGE
    assert nj.value == 0
    assert L.m16_ridge_forest_joins(N.ptr(pts), 3, N.ptr(ea), N.ptr(eb), 0, 10 ** 9, vp(ja), vp(jb),
                                    ctypes.byref(nj), N.ptr(ws), ws.numel(), N.stream_ptr()) == N.M16_OK
    assert nj.value == 2 and _set(ja[:2], jb[:2]) == {(0, 2), (0, 1)}
