"""Host steps of the sign adjustment (miccai2016_gb300/ridge_mst.py): the
vectorised sign propagation equals the reference's point-by-point loop
(adjust_directions.py:382-415) bit for bit, zero, near-zero and NaN dot
products included."""
import numpy as np
import pytest
import scipy.sparse
from scipy.sparse.csgraph import breadth_first_order, connected_components

from miccai2016_gb300.ridge_mst import propagate_signs


def _loop(n, a, b, dirs, root=0):
    """The reference's propagation, one point at a time, with the forest
    handling of propagate_signs (other trees restart at their lowest index)."""
    adjusted = np.ones((n, 3), dtype=np.float32) * np.float32(np.nan)
    g = scipy.sparse.coo_matrix((np.ones(len(a)), (a, b)), shape=(n, n)).tocsr()
    _, comp = connected_components(g, directed=False)
    _, first = np.unique(comp, return_index=True)
    starts = np.asarray([f for f in first if comp[f] != comp[root]], np.int64)
    if len(starts):
        va = np.concatenate([a, np.full(len(starts), root, np.int64)])
        vb = np.concatenate([b, starts])
        g = scipy.sparse.coo_matrix((np.ones(len(va)), (va, vb)), shape=(n, n)).tocsr()
    restart = np.zeros(n, bool)
    restart[starts] = True
    adjusted[root] = dirs[root]
    order, pred = breadth_first_order(g, root, directed=False, return_predecessors=True)
    for c in order[1:]:
        cur = dirs[c]
        if restart[c]:
            adjusted[c] = cur
            continue
        ref = adjusted[pred[c]]
        adjusted[c] = cur if np.dot(cur, ref) >= 0 else -cur
    return adjusted


@pytest.mark.parametrize("seed", range(12))
def test_vectorised_propagation_equals_the_loop(seed):
    rng = np.random.RandomState(seed)
    n = int(rng.choice([1, 2, 10, 700, 5000]))
    par = np.array([rng.randint(0, i) if i else 0 for i in range(n)])
    keep = rng.uniform(size=n) > 0.05              # a forest, not always one tree
    a = np.arange(1, n)[keep[1:]]
    b = par[1:][keep[1:]]
    perm = rng.permutation(n)
    a, b = perm[a].astype(np.int64), perm[b].astype(np.int64)
    dirs = rng.normal(size=(n, 3)).astype(np.float32)
    if n > 6:
        dirs[rng.randint(0, n, n // 20 + 1)] = 0.0                     # zero dots
        dirs[1], dirs[2], dirs[3] = [1, 0, 0], [0, 1, 0], [1e-8, 1, 0]  # exact and near-zero
        if seed % 3 == 0:
            dirs[4] = [np.nan, 0, 1]
    x = _loop(n, a, b, dirs)
    y = propagate_signs(n, a, b, dirs)
    assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
