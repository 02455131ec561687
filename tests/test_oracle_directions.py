"""The direction-kernel oracle (oracle/directions.c) against golden fixtures
from the reference's detect_ridges.cl / adjust_directions.cl and live against
them; the host-logic restatements (hysteresis, minimum spanning tree, ridge
cleaning) against the reference's literal algorithms.  CPU only."""
import io
import contextlib
import os
import sys

import numpy as np
import pytest
from scipy.sparse.csgraph import minimum_spanning_tree
from scipy.spatial.distance import pdist, squareform

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from oracle import adjust as A  # noqa: E402
from oracle import oracle as O  # noqa: E402
import inputs as I  # noqa: E402


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_direction_kernels_match_golden():
    d = I.directions_case()
    g = np.load(os.path.join(HERE, "golden", "directions.npz"))
    for th in (0.01, 0.3):
        assert np.array_equal(O.detect_ridges(d["resp"], d["quats"], th), g["ridge_%g" % th])
    assert np.array_equal(_bits(O.extract_main_directions(d["quats"])), _bits(g["main"]))
    assert np.array_equal(_bits(O.complete_transformations(d["vecs"])), _bits(g["complete"]))
    assert np.array_equal(_bits(O.adjust_nonridge_signs(d["vecs"], d["coords"], d["rdirs"], (1, 1, 1))),
                          _bits(g["adjust_iso"]))
    assert np.array_equal(_bits(O.adjust_nonridge_signs(d["vecs"], d["coords"], d["rdirs"], (1.5, 0.7, 1.2))),
                          _bits(g["adjust_aniso"]))


@pytest.mark.parametrize("shape", [(5, 7, 9), (16, 12, 20), (1, 6, 5)])
def test_direction_kernels_match_reference(has_ref, shape):
    if not has_ref:
        pytest.skip("reference checkout not present")
    rng = np.random.RandomState(sum(shape))
    resp = rng.uniform(0, 1, shape).astype(np.float32)
    q = I.random_squeezed(rng, shape)
    for th in (0.01, 0.5):
        assert np.array_equal(O.detect_ridges(resp, q, th), O.ref_detect_ridges(resp, q, th))
    assert np.array_equal(_bits(O.extract_main_directions(q)), _bits(O.ref_extract_main_directions(q)))
    v = rng.normal(size=shape + (3,)).astype(np.float32)
    assert np.array_equal(_bits(O.complete_transformations(v)), _bits(O.ref_complete_transformations(v)))
    R = 17
    coords = np.stack([rng.randint(0, s, R) for s in shape], -1).astype(np.uint16)
    rd = rng.normal(size=(R, 3)).astype(np.float32)
    for sc in [(1, 1, 1), (0.5, 2.0, 1.25)]:
        assert np.array_equal(_bits(O.adjust_nonridge_signs(v, coords, rd, sc)),
                              _bits(O.ref_adjust_nonridge_signs(v, coords, rd, sc)))


def test_label_hysteresis_equals_the_reference_flood_fill():
    from miccai2016_gb300.ridge_detection import hysteresis_threshold
    rng = np.random.RandomState(2)
    for t in range(30):
        shape = tuple(rng.randint(3, 14, 3))
        cand = rng.uniform(size=shape) < rng.uniform(0.1, 0.5)
        sure = cand & (rng.uniform(size=shape) < 0.1)
        if t % 5 == 0:
            sure |= rng.uniform(size=shape) < 0.02   # sure voxels outside the candidates
        a = A.hysteresis_threshold(cand.copy(), sure.copy())
        b = hysteresis_threshold(cand.copy(), sure.copy(), labeler="host")
        assert np.array_equal(a, b)


def test_stable_mst_is_scipys_tree_when_distances_are_distinct():
    rng = np.random.RandomState(3)
    for _ in range(5):
        pts = rng.uniform(0, 50, (300, 3))
        d = pdist(pts)
        assert len(np.unique(d)) == len(d)
        ref = minimum_spanning_tree(squareform(d)).tocoo()
        ours = A.stable_mst(pts, (1, 1, 1)).tocoo()
        e1 = set(zip(np.minimum(ref.row, ref.col), np.maximum(ref.row, ref.col)))
        e2 = set(zip(np.minimum(ours.row, ours.col), np.maximum(ours.row, ours.col)))
        assert e1 == e2


@pytest.mark.parametrize("vs", [(1, 1, 1), (1.5, 0.7, 1.2), (1, 1, 3)])
def test_sparse_mst_equals_the_dense_stable_kruskal(vs):
    from miccai2016_gb300.ridge_mst import ridge_mst_edges
    rng = np.random.RandomState(int(sum(vs) * 10))
    for _ in range(4):
        pts = np.unique(np.concatenate([rng.randint(0, 10, (120, 3)) + rng.randint(0, 35, 3) for _ in range(4)]), axis=0)
        pts = pts[rng.permutation(len(pts))]
        a, b = ridge_mst_edges(pts, vs, local="host")
        t = A.stable_mst(pts, vs).tocoo()
        assert set(zip(np.minimum(a, b), np.maximum(a, b))) == set(zip(np.minimum(t.row, t.col),
                                                                       np.maximum(t.row, t.col)))


@pytest.mark.parametrize("vs", [(1, 1, 1), (1, 1, 2.5)])
def test_join_of_one_large_and_many_small_trees_equals_the_dense_stable_kruskal(vs):
    """Trees of very different sizes, in index orders that put the large one
    first, last and in between: the join queries the smaller tree of every
    pair against the larger one."""
    from miccai2016_gb300.ridge_mst import ridge_mst_edges
    rng = np.random.RandomState(7)
    for t in range(3):
        big = np.argwhere(np.ones((9, 9, 6), bool))
        small = [rng.randint(0, 3, (rng.randint(1, 5), 3)) + rng.randint(-12, 24, 3) for _ in range(12)]
        pts = np.unique(np.concatenate([big] + small), axis=0)
        order = [rng.permutation(len(pts)), np.argsort(-np.abs(pts).sum(1), kind="stable"),
                 np.argsort(np.abs(pts - 4).sum(1), kind="stable")][t]
        pts = pts[order]
        a, b = ridge_mst_edges(pts, vs, local="host")
        ref = A.stable_mst(pts, vs).tocoo()
        assert set(zip(np.minimum(a, b), np.maximum(a, b))) == set(zip(np.minimum(ref.row, ref.col),
                                                                       np.maximum(ref.row, ref.col)))


def test_forest_components_number_like_scipy():
    import scipy.sparse
    from scipy.sparse.csgraph import connected_components
    from miccai2016_gb300.ridge_mst import forest_components
    rng = np.random.RandomState(8)
    n = 500
    p = rng.permutation(n)
    a, b = [], []
    for k in range(1, n):
        if rng.uniform() < 0.9:   # a random forest: each point hangs off an earlier one, or starts a tree
            a.append(p[k]); b.append(p[rng.randint(0, k)])
    a, b = np.asarray(a), np.asarray(b)
    n1, c1 = forest_components(n, a, b)
    n2, c2 = connected_components(scipy.sparse.coo_matrix((np.ones(len(a)), (a, b)), shape=(n, n)), directed=False)
    assert n1 == n2 and np.array_equal(c1, c2)


def test_ridge_directions_and_cleaning_match_the_reference_logic():
    from miccai2016_gb300.adjust_directions import AdvancedAdjuster
    rng = np.random.RandomState(4)
    shape = (24, 24, 24)
    ridge = np.zeros(shape, np.float32)
    # a few short 26-connected curves and specks
    for _ in range(6):
        p = rng.randint(2, 22, 3)
        for _ in range(rng.randint(1, 25)):
            ridge[tuple(np.clip(p, 0, 23))] = 1
            p = p + rng.randint(-1, 2, 3)
    main = rng.normal(size=shape + (3,)).astype(np.float32)
    obj = AdvancedAdjuster((0.01, 0.3), np.zeros(shape + (3,), np.float32), np.zeros(shape, np.float32))
    obj.mst_local = "host"
    obj.labeler = "host"
    c1, d1 = A.adjust_ridge_directions(ridge, main, (1.0, 1.0, 1.0))
    c2, d2 = obj._adjust_ridge_directions(ridge, main)
    assert np.array_equal(c1, c2) and np.array_equal(_bits(d1), _bits(d2))
    with contextlib.redirect_stdout(io.StringIO()):
        k1 = A.clean_ridge(ridge, c1, d1, (1.0, 1.0, 1.0))
        k2 = obj._do_clean_ridge(ridge, c2, d2)
    assert np.array_equal(k1, k2)


def test_cleaning_is_the_same_without_joining_the_segments():
    from miccai2016_gb300.adjust_directions import AdvancedAdjuster
    rng = np.random.RandomState(11)
    shape = (30, 30, 30)
    ridge = np.zeros(shape, np.float32)
    for _ in range(12):
        p = rng.randint(2, 28, 3)
        for _ in range(rng.randint(1, 30)):
            ridge[tuple(np.clip(p, 0, 29))] = 1
            p = p + rng.randint(-1, 2, 3)
    main = rng.normal(size=shape + (3,)).astype(np.float32)
    obj = AdvancedAdjuster((0.01, 0.3), np.zeros(shape + (3,), np.float32), np.zeros(shape, np.float32))
    obj.mst_local = "host"
    obj.labeler = "host"
    c1, d1 = obj._adjust_ridge_directions(ridge, main, join_components=True)
    c2, d2 = obj._adjust_ridge_directions(ridge, main, join_components=False)
    with contextlib.redirect_stdout(io.StringIO()):
        k1 = A.clean_ridge(ridge, c1, d1, (1.0, 1.0, 1.0))
        k2 = obj._do_clean_ridge(ridge, c2, d2)
    assert np.array_equal(k1, k2)
    # every point's direction is the joined one up to one sign per segment
    assert np.allclose(np.abs(d1), np.abs(d2))


def test_cleaning_of_a_ridge_without_background_drops_label_one_like_the_reference():
    """np.unique(components)[1:] drops label 1 when no voxel is background."""
    from miccai2016_gb300.adjust_directions import AdvancedAdjuster
    rng = np.random.RandomState(12)
    shape = (3, 4, 5)
    ridge = np.ones(shape, np.float32)
    main = rng.normal(size=shape + (3,)).astype(np.float32)
    obj = AdvancedAdjuster((0.01, 0.3), np.zeros(shape + (3,), np.float32), np.zeros(shape, np.float32))
    obj.mst_local = "host"
    obj.labeler = "host"
    c, d = obj._adjust_ridge_directions(ridge, main)
    with contextlib.redirect_stdout(io.StringIO()):
        k1 = A.clean_ridge(ridge, c, d, (1.0, 1.0, 1.0))
        k2 = obj._do_clean_ridge(ridge, c, d)
    assert np.array_equal(k1, k2) and not k2.any()


@pytest.mark.parametrize("n,voxel_size", [(300, (1, 1, 1)), (900, (1, 1, 1)), (600, (1.5, 0.7, 2.0)), (1, (1, 1, 1))])
def test_prim_mst_is_the_stable_kruskal_tree(n, voxel_size):
    """The oracle's O(R) memory tree (Prim under the (distance, i, j) order)
    equals the dense stable Kruskal tree on lattice points full of ties."""
    from oracle import adjust as A
    rng = np.random.RandomState(n)
    pts = sorted(set(tuple(p) for p in rng.randint(0, 11, (n, 3))))
    a, b = A.stable_mst(pts, voxel_size), A.prim_mst(pts, voxel_size)
    ea = set(tuple(sorted(e)) for e in zip(*a.nonzero()))
    eb = set(tuple(sorted(e)) for e in zip(*b.nonzero()))
    assert len(eb) == len(pts) - 1 and ea == eb
