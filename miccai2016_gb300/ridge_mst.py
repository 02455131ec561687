"""
Minimum spanning tree over ridge points without the reference's O(R^2)
distance matrix.

The reference builds the dense distance matrix of all R ridge points
(pdist + squareform) and hands it to SciPy's minimum_spanning_tree
(src/processing/adjust_directions.py:374-379), i.e. Kruskal's algorithm over
all R(R-1)/2 pairs.  Equal distances are everywhere on a voxel grid; SciPy
orders them with an unstable argsort, so the reference's tree among
equal-weight alternatives is an accident of the sorting implementation.  This
module defines the order as (weight, i, j) with i < j -- what SciPy's Kruskal
gives with a stable sort of the condensed distances -- and computes that exact
tree in O(R log R):

1. local phase: every pair whose offset has a scaled length <= r (r = the
   length of the (1, 1, 1) offset, so all 26-neighbours are included) is a
   candidate; Kruskal over the candidates in (weight, i, j) order.  Every
   edge not longer than r is a candidate, so this reproduces the full
   Kruskal up to weight r;
2. global phase: the remaining trees are joined like the full Kruskal would
   join them -- by Kruskal over, for each pair of trees, their least edge in
   (weight, i, j) order, found exactly with k-d trees.

Weights are computed as pdist computes them: sqrt of the sum over the axes of
the squared differences of the scaled coordinates, in float64.
"""
from __future__ import annotations

import itertools

import numpy as np
import scipy.sparse
from scipy.sparse.csgraph import breadth_first_order, connected_components, minimum_spanning_tree
from scipy.spatial import cKDTree


def _weights(u, i, j):
    d = u[i] - u[j]
    return np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])


def _kruskal_by_order(n, i, j, order_keys):
    """Kruskal over edges (i, j) taken in the lexicographic order of
    order_keys (tuple for np.lexsort, last key primary).  The order is turned
    into distinct ranks so SciPy's Kruskal has no ties left to break."""
    if len(i) == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    order = np.lexsort(order_keys)
    rank = np.empty(len(order), np.float64)
    rank[order] = np.arange(1, len(order) + 1, dtype=np.float64)
    g = scipy.sparse.coo_matrix((rank, (i, j)), shape=(n, n)).tocsr()
    t = minimum_spanning_tree(g).tocoo()
    return t.row.astype(np.int64), t.col.astype(np.int64)


def ridge_mst_edges(points, voxel_size=(1.0, 1.0, 1.0), join_components=True):
    """Edges (a, b) of the (weight, i, j)-ordered Euclidean MST of integer
    points (R x 3, axis order 0, 1, 2) with per-axis voxel size.  With
    join_components=False only the local phase runs: the result is the MST
    minus its edges longer than r, i.e. a spanning tree of every group of
    points linked by steps not longer than r (each 26-connected set lies in
    one such group)."""
    pts = np.asarray(points, dtype=np.int64)
    R = len(pts)
    if R < 2:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    vs = np.asarray(np.multiply(np.ones(3), voxel_size), np.float64)
    u = np.multiply(pts, vs)   # the coordinates pdist sees
    r = float(np.sqrt(np.sum(vs * vs)))
    # all integer offsets with scaled length <= r, one of each +-pair
    ext = [int(np.floor(r / vs[k] + 1e-9)) for k in range(3)]
    offsets = []
    for off in itertools.product(*[range(-e, e + 1) for e in ext]):
        if off <= (0, 0, 0):
            continue
        if np.sqrt(sum((off[k] * vs[k]) ** 2 for k in range(3))) <= r * (1 + 1e-12):
            offsets.append(off)
    lo = pts.min(0)
    dims = pts.max(0) - lo + 1
    grid = np.full(tuple(int(d) for d in dims), -1, np.int64)
    q = pts - lo
    grid[q[:, 0], q[:, 1], q[:, 2]] = np.arange(R)
    ii, jj = [], []
    for off in offsets:
        t = q + np.asarray(off)
        ok = np.all((t >= 0) & (t < dims), axis=1)
        src = np.nonzero(ok)[0]
        dst = grid[t[ok, 0], t[ok, 1], t[ok, 2]]
        m = dst >= 0
        a, b = src[m], dst[m]
        ii.append(np.minimum(a, b))
        jj.append(np.maximum(a, b))
    i = np.concatenate(ii) if ii else np.zeros(0, np.int64)
    j = np.concatenate(jj) if jj else np.zeros(0, np.int64)
    w = _weights(u, i, j)
    keep = w <= r   # exactly the edges not longer than r
    i, j, w = i[keep], j[keep], w[keep]
    ta, tb = _kruskal_by_order(R, i, j, (j, i, w))
    # global phase: join the local trees
    forest = scipy.sparse.coo_matrix((np.ones(len(ta)), (ta, tb)), shape=(R, R))
    ncomp, comp = connected_components(forest, directed=False)
    if ncomp == 1 or not join_components:
        return ta, tb
    members = [np.nonzero(comp == c)[0] for c in range(ncomp)]
    trees = [cKDTree(u[m]) for m in members]
    ci, cj, cw, ca, cb = [], [], [], [], []
    for A in range(ncomp):
        mA = members[A]
        for B in range(A + 1, ncomp):
            mB = members[B]
            # nearest point of A for each point of B, then every pair at that
            # distance, so ties resolve by (i, j)
            dist, _ = trees[A].query(u[mB], k=1)
            dmin = float(np.min(dist))
            cand = trees[A].query_ball_point(u[mB], dmin * (1 + 1e-9) + 1e-12)
            pa, pb = [], []
            for kb, lst in enumerate(cand):
                for ka in lst:
                    pa.append(mA[ka])
                    pb.append(mB[kb])
            pa = np.asarray(pa, np.int64)
            pb = np.asarray(pb, np.int64)
            lo_, hi_ = np.minimum(pa, pb), np.maximum(pa, pb)
            ww = _weights(u, lo_, hi_)
            best = np.lexsort((hi_, lo_, ww))[0]
            ci.append(A); cj.append(B); cw.append(ww[best]); ca.append(lo_[best]); cb.append(hi_[best])
    ci, cj = np.asarray(ci), np.asarray(cj)
    cw, ca, cb = np.asarray(cw), np.asarray(ca), np.asarray(cb)
    ga, gb = _kruskal_by_order(ncomp, ci, cj, (cb, ca, cw))
    # map the chosen component pairs back to their point pairs
    pair = {(int(x), int(y)): k for k, (x, y) in enumerate(zip(ci, cj))}
    sel = [pair[(int(min(x, y)), int(max(x, y)))] for x, y in zip(ga, gb)]
    return np.concatenate([ta, ca[sel]]), np.concatenate([tb, cb[sel]])


def propagate_signs(n, edges_a, edges_b, dirs, root=0):
    """Sign propagation along the tree from `root` (adjust_directions.py:382-415):
    a child keeps its direction if its dot product with its parent's adjusted
    direction is >= 0, else it is negated.  When the edges form a forest,
    every other tree is propagated from its lowest-index point, as if that
    point were the root."""
    adjusted = np.ones((n, 3), dtype=np.float32) * np.float32(np.nan)
    g = scipy.sparse.coo_matrix((np.ones(len(edges_a)), (edges_a, edges_b)), shape=(n, n)).tocsr()
    ncomp, comp = connected_components(g, directed=False)
    # the other trees hang off `root` through virtual edges to their
    # lowest-index points, which restart the propagation
    _, first = np.unique(comp, return_index=True)
    starts = np.asarray([f for f in first if comp[f] != comp[root]], np.int64)
    if len(starts):
        va = np.concatenate([edges_a, np.full(len(starts), root, np.int64)])
        vb = np.concatenate([edges_b, starts])
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
