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

import ctypes
import itertools

import numpy as np
import scipy.sparse
from scipy.sparse.csgraph import minimum_spanning_tree
from scipy.spatial import cKDTree

from . import _native as N


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


def _local_offsets(vs):
    """r = |voxel size| and every integer offset (one of each +- pair, the
    lexicographically positive one) with scaled length <= r."""
    r = float(np.sqrt(np.sum(vs * vs)))
    ext = [int(np.floor(r / vs[k] + 1e-9)) for k in range(3)]
    offsets = []
    for off in itertools.product(*[range(-e, e + 1) for e in ext]):
        if off <= (0, 0, 0):
            continue
        if np.sqrt(sum((off[k] * vs[k]) ** 2 for k in range(3))) <= r * (1 + 1e-12):
            offsets.append(off)
    return r, offsets


def _local_mst_host(pts, vs, r, offsets):
    """The local phase on the host: Kruskal over the candidate edges in
    (weight, i, j) order."""
    R = len(pts)
    u = np.multiply(pts, vs)   # the coordinates pdist sees
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
    return _kruskal_by_order(R, i, j, (j, i, w))


def _local_mst_gpu(pts, vs, r, offsets, keep_device=False):
    """The local phase on the GPU (m16_ridge_mst_local, Boruvka rounds in the
    same (weight, i, j) order): the same edge set as _local_mst_host.  With
    keep_device, also the device points (int32 R x 3) and edges (int32 E x 2)."""
    d_pts, d_edges = _local_mst_device(pts, vs, r, offsets)
    e = d_edges.cpu().numpy().astype(np.int64)
    if keep_device:
        return e[:, 0], e[:, 1], d_pts, d_edges
    return e[:, 0], e[:, 1]


def _local_mst_device(pts, vs, r, offsets, d_points=None, box=None):
    """_local_mst_gpu's device arrays: the points (int32 R x 3) and the
    local forest's edges (int32 E x 2), nothing copied back.  d_points: the
    same points already on the device (any integer dtype); box: (lo, dims)
    of a box holding them (else their bounding box, from the host points)."""
    torch = N.torch_mod()
    L = N.lib()
    R = len(pts)
    if d_points is not None:
        d_pts = d_points.to(device=N.device(), dtype=torch.int32).contiguous()
    else:
        p32 = np.ascontiguousarray(pts, np.int32)
        d_pts = torch.from_numpy(p32).to(N.device())
    if box is not None:
        lo = np.ascontiguousarray(box[0], np.int32)
        dims = np.ascontiguousarray(box[1], np.int32)
    else:
        p32 = np.ascontiguousarray(pts, np.int32)
        # per column: an axis-0 reduction of an R x 3 array is several times slower
        lo = np.array([p32[:, k].min() for k in range(3)], np.int32)
        dims = np.array([p32[:, k].max() for k in range(3)], np.int32) - lo + 1
    offs = np.ascontiguousarray(np.asarray(offsets, np.int32).reshape(-1, 3))
    edges = torch.empty((max(R - 1, 1), 2), dtype=torch.int32, device=N.device())
    ws = N.workspace(L.m16_ridge_mst_workspace_bytes(R, dims.ctypes.data_as(ctypes.c_void_p), len(offs)))
    vsc = (ctypes.c_double * 3)(*[float(v) for v in vs])
    ne = ctypes.c_int64(0)
    st = L.m16_ridge_mst_local(N.ptr(d_pts), R, lo.ctypes.data_as(ctypes.c_void_p),
                               dims.ctypes.data_as(ctypes.c_void_p), vsc, offs.ctypes.data_as(ctypes.c_void_p),
                               len(offs), float(r), N.ptr(edges), ctypes.byref(ne), N.ptr(ws), ws.numel(),
                               N.stream_ptr())
    N.check("m16_ridge_mst_local", st)
    return d_pts, edges[:ne.value]


# pair evaluations above which the joins stay on the host (k-d trees)
JOIN_MAX_PAIR_EVALUATIONS = 40_000_000_000


def _joins_gpu(d_pts, d_edges):
    """The joins of the local trees on the device (m16_ridge_forest_joins) for
    unit voxel size: (a, b) host arrays of the joining edges, or None where
    the exact search would take more than JOIN_MAX_PAIR_EVALUATIONS distance
    evaluations (then the host joins them)."""
    L = N.lib()
    R = int(d_pts.shape[0])
    ea = d_edges[:, 0].contiguous()
    eb = d_edges[:, 1].contiguous()
    ja = np.empty(max(R - 1, 1), np.int32)
    jb = np.empty(max(R - 1, 1), np.int32)
    nj = ctypes.c_int64(0)
    ws = N.workspace(L.m16_ridge_forest_joins_workspace_bytes(R))
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    st = L.m16_ridge_forest_joins(N.ptr(d_pts), R, N.ptr(ea), N.ptr(eb), int(ea.numel()),
                                  JOIN_MAX_PAIR_EVALUATIONS, vp(ja), vp(jb), ctypes.byref(nj), N.ptr(ws), ws.numel(),
                                  N.stream_ptr())
    if st == N.M16_ERR_TOO_LARGE:
        return None
    N.check("m16_ridge_forest_joins", st)
    return ja[:nj.value].astype(np.int64), jb[:nj.value].astype(np.int64)


def forest_components(n, ea, eb):
    """(count, component of each point) of the forest with edges (ea, eb) on
    points 0..n-1, numbered in the order of each component's lowest index --
    the numbering of scipy.sparse.csgraph.connected_components.  The
    components come from the library's traversal (m16_tree_order): it starts
    a new tree at each point not yet reached, in index order."""
    L = N.lib()
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    a32 = np.ascontiguousarray(ea, dtype=np.int32)
    b32 = np.ascontiguousarray(eb, dtype=np.int32)
    order = np.empty(n, np.int32)
    pred = np.empty(n, np.int32)
    N.check("m16_tree_order", L.m16_tree_order(n, vp(a32), vp(b32), len(a32), 0, vp(order), vp(pred)))
    starts = pred[order] < 0
    comp = np.empty(n, np.int64)
    comp[order] = np.cumsum(starts) - 1
    return int(np.count_nonzero(starts)), comp


def ridge_mst_edges(points, voxel_size=(1.0, 1.0, 1.0), join_components=True, local="gpu", joins_on_device=True,
                    on_device=False, d_points=None, box=None):
    """Edges (a, b) of the (weight, i, j)-ordered Euclidean MST of integer
    points (R x 3, axis order 0, 1, 2, distinct) with per-axis voxel size.
    With join_components=False only the local phase runs: the result is the
    MST minus its edges longer than r, i.e. a spanning tree of every group of
    points linked by steps not longer than r (each 26-connected set lies in
    one such group).  local selects where the local phase runs ("gpu", the
    default, or "host"); both give the same edges.  With the local phase on
    the GPU and unit voxel size, the trees are joined on the device too
    (m16_ridge_forest_joins, exact in integer arithmetic) unless
    joins_on_device is False; otherwise k-d trees on the host join them.
    With on_device, where the edges are all known on the device (the local
    phase there, and no joins or the device's) they stay there: (a, b) are
    then CUDA int32 tensors; otherwise host int64 arrays.  d_points (the
    same points as a CUDA tensor) and box ((lo, dims) of a box holding them,
    e.g. the volume's) spare the local phase on the GPU its upload and its
    bounding box; a point outside the box fails the call."""
    pts = np.asarray(points)
    if pts.dtype.kind not in "iu":
        pts = pts.astype(np.int64)
    R = len(pts)
    if R < 2:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    vs = np.asarray(np.multiply(np.ones(3), voxel_size), np.float64)
    r, offsets = _local_offsets(vs)
    if local == "gpu":
        d_pts, d_edges = _local_mst_device(pts, vs, r, offsets, d_points=d_points, box=box)

        def host_edges():
            e = d_edges.cpu().numpy().astype(np.int64)
            return e[:, 0], e[:, 1]

        if not join_components or int(d_edges.shape[0]) == R - 1:   # not asked for, or already one tree
            return (d_edges[:, 0].contiguous(), d_edges[:, 1].contiguous()) if on_device else host_edges()
        if np.all(vs == 1.0) and joins_on_device:
            j = _joins_gpu(d_pts, d_edges)
            if j is not None:
                if on_device:
                    torch = N.torch_mod()
                    up = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.int32)).to(d_edges.device)
                    return torch.cat([d_edges[:, 0], up(j[0])]), torch.cat([d_edges[:, 1], up(j[1])])
                ta, tb = host_edges()
                return np.concatenate([ta, j[0]]), np.concatenate([tb, j[1]])
        ta, tb = host_edges()
    elif local == "host":
        pts = pts.astype(np.int64)
        ta, tb = _local_mst_host(pts, vs, r, offsets)
        # global phase: join the local trees
        if not join_components or len(ta) == R - 1:   # not asked for, or already one tree
            return ta, tb
    else:
        raise ValueError("local must be 'gpu' or 'host'")
    u = np.multiply(pts.astype(np.int64), vs)   # the coordinates pdist sees (host joins only)
    ncomp, comp = forest_components(R, ta, tb)
    by_comp = np.argsort(comp, kind="stable")   # each component's points in index order
    members = np.split(by_comp, np.cumsum(np.bincount(comp, minlength=ncomp))[:-1])
    trees = {}

    def tree(c):
        # kd-trees only find candidates (their queries are exact); the
        # sliding-midpoint build is the fastest one
        if c not in trees:
            trees[c] = cKDTree(u[members[c]], balanced_tree=False, compact_nodes=False)
        return trees[c]

    ci, cj, cw, ca, cb = [], [], [], [], []
    for A in range(ncomp):
        for B in range(A + 1, ncomp):
            # the smaller tree's points are queried against the larger one:
            # nearest point for each, then every pair at the least distance,
            # so ties resolve by (i, j)
            S, Lg = (A, B) if len(members[A]) <= len(members[B]) else (B, A)
            mS, mL = members[S], members[Lg]
            dist, _ = tree(Lg).query(u[mS], k=1)
            dmin = float(np.min(dist))
            near = np.nonzero(dist <= dmin * (1 + 1e-9) + 1e-12)[0]
            cand = tree(Lg).query_ball_point(u[mS[near]], dmin * (1 + 1e-9) + 1e-12)
            ps = np.repeat(mS[near], [len(lst) for lst in cand])
            pl = mL[np.fromiter(itertools.chain.from_iterable(cand), np.int64)]
            lo_, hi_ = np.minimum(ps, pl), np.maximum(ps, pl)
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


def _dot_signs(cur, par):
    """Sign (-1, 0, +1; 2 for NaN) of np.dot(cur[k], par[k]) for every row k,
    exactly as the per-row float32 np.dot of the reference's loop rounds it.
    The float64 sum of the three (exact) float64 products has the sign of the
    exact dot product; np.dot's float32 result can only differ from it when
    the exact value lies within its rounding error of zero, and only those
    rows are evaluated with np.dot itself."""
    c64 = cur.astype(np.float64)
    p64 = par.astype(np.float64)
    prod = c64 * p64
    exact = prod[:, 0] + prod[:, 1] + prod[:, 2]
    nan = np.isnan(exact)
    sign = np.sign(np.where(nan, 0.0, exact)).astype(np.int8)
    sign[nan] = 2   # NaN: "np.dot(...) >= 0" fails, the point is negated whatever its parent's sign
    # float32 sum of three products: error below 3 * 2^-23 * sum |products|
    # (generous: covers contraction into fused multiply-adds too)
    bound = 8.0 * 2.0 ** -23 * np.sum(np.abs(prod), axis=1)
    unsure = np.nonzero(np.abs(exact) <= bound)[0]
    for k in unsure:
        d = np.dot(cur[k], par[k])
        sign[k] = 1 if d > 0 else (-1 if d < 0 else 0)
    return sign


def propagate_signs(n, edges_a, edges_b, dirs, root=0):
    """Sign propagation along the tree from `root` (adjust_directions.py:382-415):
    a child keeps its direction if its dot product with its parent's adjusted
    direction is >= 0, else it is negated.  When the edges form a forest,
    every other tree is propagated from its lowest-index point, as if that
    point were the root.

    The reference visits the points one by one.  Here all decisions are
    evaluated at once: the visiting order and parents come from one traversal
    (m16_tree_order), and with s the sign a point's direction ends up with,
    np.dot(d_c, s_p d_p) = s_p np.dot(d_c, d_p) bit for bit (negating one
    operand negates every rounded step), so s_c = +1 where np.dot(d_c, d_p)
    is zero (either sign of zero passes ">= 0"), s_c = -1 where it is NaN,
    and s_c = s_p sign(np.dot(d_c, d_p)) elsewhere; the signs are then
    composed in one pass in visiting order (m16_compose_signs, host code of
    the library)."""
    dirs = np.asarray(dirs, dtype=np.float32)
    adjusted = np.ones((n, 3), dtype=np.float32) * np.float32(np.nan)
    L = N.lib()
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    ea = np.ascontiguousarray(edges_a, dtype=np.int32)
    eb = np.ascontiguousarray(edges_b, dtype=np.int32)
    order = np.empty(n, np.int32)
    pred = np.empty(n, np.int32)
    N.check("m16_tree_order", L.m16_tree_order(n, vp(ea), vp(eb), len(ea), int(root), vp(order), vp(pred)))
    e = np.zeros(n, dtype=np.int8)            # 0: keeps its direction (the root and each tree's first point)
    kids = np.nonzero(pred >= 0)[0]
    e[kids] = _dot_signs(dirs[kids], dirs[pred[kids].astype(np.int64)])
    # one pass in visiting order: s_c = s_parent * e_c (+1 at zero dots, -1 at NaN dots)
    sgn = np.ones(n, dtype=np.int8)
    N.check("m16_compose_signs", L.m16_compose_signs(n, vp(order), n, vp(pred), vp(e), vp(sgn)))
    val = sgn
    neg = val[:, None] < 0
    adjusted[:] = np.where(neg, -dirs, dirs)   # negation flips the sign bit, NaN too
    return adjusted


def propagate_signs_device(d_dirs, edges_a, edges_b):
    """propagate_signs from root 0 on the device: d_dirs (CUDA float32
    tensor, n x 3), the forest's edges (host or device int arrays).  Every
    edge's dot-product sign comes from m16_ridge_edge_codes; the few whose
    float32 rounding could decide the sign are evaluated with np.dot itself,
    as the reference's loop evaluates them; m16_ridge_signs composes the signs
    (a parity union-find over the +-1 edges).  Returns the adjusted
    directions as a CUDA tensor, bit for bit propagate_signs(n, a, b, dirs)."""
    torch = N.torch_mod()
    L = N.lib()
    n = int(d_dirs.shape[0])
    dev = d_dirs.device
    d_dirs = d_dirs.contiguous()
    to_dev = lambda e: (e.to(device=dev, dtype=torch.int32).contiguous() if N.is_torch(e)
                        else torch.from_numpy(np.ascontiguousarray(e, dtype=np.int32)).to(dev))
    d_a, d_b = to_dev(edges_a), to_dev(edges_b)
    ne = int(d_a.numel())
    codes = torch.empty(max(ne, 1), dtype=torch.int8, device=dev)
    N.check("m16_ridge_edge_codes", L.m16_ridge_edge_codes(N.ptr(d_dirs), n, N.ptr(d_a), N.ptr(d_b), ne,
                                                           N.ptr(codes), N.stream_ptr()))
    unsure = torch.nonzero(codes[:ne] == 3).flatten()
    if unsure.numel():
        ca = d_dirs[d_a[unsure].long()].cpu().numpy()
        cb = d_dirs[d_b[unsure].long()].cpu().numpy()
        fixed = np.empty(len(ca), np.int8)
        for k in range(len(ca)):
            d = np.dot(ca[k], cb[k])   # the float32 np.dot of the reference's loop (commutative)
            fixed[k] = 1 if d > 0 else (-1 if d < 0 else 0)
        codes[unsure] = torch.from_numpy(fixed).to(dev)
    signs = torch.empty(n, dtype=torch.int8, device=dev)
    ws = N.workspace(L.m16_ridge_signs_workspace_bytes(n, ne))
    N.check("m16_ridge_signs", L.m16_ridge_signs(n, N.ptr(d_a), N.ptr(d_b), N.ptr(codes), ne, N.ptr(signs), N.ptr(ws),
                                                 ws.numel(), N.stream_ptr()))
    # negate by flipping the sign bit, as numpy's unary minus does (NaN
    # included: arithmetic on the GPU would return the canonical NaN)
    flip = torch.where(signs[:, None] < 0, torch.tensor(-2 ** 31, dtype=torch.int32, device=dev),
                       torch.tensor(0, dtype=torch.int32, device=dev))
    return torch.bitwise_xor(d_dirs.view(torch.int32), flip).view(torch.float32)
