"""
oracle/adjust.py -- the reference's direction-adjustment host logic restated
in Python 3 over the oracle's C kernels (TEST INFRASTRUCTURE ONLY).

Follows src/processing/adjust_directions.py:213-446 and
src/processing/ridge_detection.py:80-131 literally: the stack-based hysteresis
flood fill, the per-label loop of the ridge cleaning, SciPy's minimum spanning
tree (with equal distances in (i, j) order, see stable_mst) and the
depth-first sign propagation.
"""
from __future__ import annotations

import numpy as np
from scipy.ndimage import label
from scipy.sparse import csr_matrix
from scipy.sparse.csgraph import minimum_spanning_tree
from scipy.spatial.distance import pdist, squareform

from . import oracle as O


def hysteresis_threshold(cand, sure):
    """ridge_detection.py:80-131 (stack flood fill over the 26-neighbourhood)."""
    assert cand.shape == sure.shape

    def find_neighbors(pos, cand):
        lower = np.maximum(0, np.subtract(pos, 1))
        hood = cand[lower[0]:pos[0] + 2, lower[1]:pos[1] + 2, lower[2]:pos[2] + 2]
        nb = list(zip(*np.where(hood)))
        if nb:
            nb = [tuple(n) for n in (lower + np.asarray(nb))]
        return nb

    stack = list(zip(*np.where(sure)))
    while stack:
        c = stack.pop()
        sure[c] = True
        cand[c] = False
        stack.extend(find_neighbors(c, cand))
    return sure


def stable_mst(points, voxel_size):
    """The reference's minimum_spanning_tree(squareform(pdist(...)))
    (adjust_directions.py:376-379) with the condensed distances ranked by a
    stable sort, so equal distances are taken in (i, j) order (SciPy itself
    uses an unstable argsort there, whose tie order depends on the numpy
    build).  Returns the tree as a CSR matrix."""
    dists = pdist(np.multiply(points, voxel_size), "euclidean")
    order = np.argsort(dists, kind="stable")
    rank = np.empty(len(dists), np.float64)
    rank[order] = np.arange(1, len(dists) + 1, dtype=np.float64)
    return csr_matrix(minimum_spanning_tree(squareform(rank), overwrite=True))


# above this many ridge points the dense R x R matrix of stable_mst is too
# large, and prim_mst computes the same tree
DENSE_MST_MAX_POINTS = 3000


def prim_mst(points, voxel_size):
    """The tree of stable_mst without the R x R matrix: Prim's algorithm under
    the total order (distance, min(i, j), max(i, j)) of the edges, which is
    the order stable_mst ranks them in.  Under a strict total order the
    minimum spanning tree is unique, so Prim's and Kruskal's give the same
    edge set.  The distances are pdist's: the square root of the summed
    squared coordinate differences of the scaled points, in float64.
    Returns the tree as a CSR matrix (one entry per edge)."""
    pts = np.multiply(np.asarray(points, np.float64), voxel_size).reshape(-1, 3)
    n = len(pts)
    rows, cols = O.prim_mst_edges(pts)
    return csr_matrix((np.ones(len(rows)), (rows, cols)), shape=(n, n))


def adjust_ridge_directions(labeled_ridge, main_dirs, voxel_size):
    """adjust_directions.py:365-417 (with the stable tree of stable_mst, or
    the same tree from prim_mst for many points)"""
    i_ridge = list(zip(*np.where(labeled_ridge)))
    mst = (stable_mst if len(i_ridge) <= DENSE_MST_MAX_POINTS else prim_mst)(i_ridge, voxel_size)
    adjusted = np.ones_like(i_ridge, dtype=np.float32) * np.float32(np.nan)
    adjusted[0] = main_dirs[i_ridge[0]]
    get_children = lambda i: np.r_[mst[i].nonzero()[1], mst[:, i].nonzero()[0]]
    visited = lambda i: not np.isnan(adjusted[i, 0])
    adjust = lambda cur, ref: cur if np.dot(cur, ref) >= 0 else -cur
    stack = [0]
    while stack:
        i = stack.pop()
        dir_i = adjusted[i]
        for child in get_children(i):
            if not visited(child):
                adjusted[child] = adjust(main_dirs[i_ridge[child]], dir_i)
                stack.append(child)
    return np.asarray(i_ridge, dtype=np.uint16, order="C"), adjusted


def clean_ridge(labeled_ridge, ridge_coords, ridge_dirs, voxel_size):
    """adjust_directions.py:290-339"""
    scaled_dirs = ridge_dirs * tuple(voxel_size)
    dirs_dict = {tuple(c): d for (c, d) in zip(ridge_coords, scaled_dirs)}
    components = label(labeled_ridge, structure=np.ones((3, 3, 3), dtype=int))[0]
    labels = np.unique(components)[1:]
    lengths = {}
    for lab in labels:
        dirs = [dirs_dict[tuple(i)] for i in np.array(np.where(components == lab)).T]
        lengths[lab] = np.linalg.norm(np.sum(dirs, axis=0))
    sorted_labels = sorted(lengths, key=lambda k: lengths[k], reverse=True)
    boundary = int(np.ceil(3 * np.log(np.e + len(sorted_labels))))
    kept = sorted_labels[:boundary]
    return np.isin(components, kept).astype(labeled_ridge.dtype).reshape(components.shape)


def advanced_adjuster(qeigs, response, threshold=(0.01, 0.3), voxel_size=(1, 1, 1), ridge_detection_only=False,
                      clean=True, stages=None):
    """AdvancedAdjuster.execute (adjust_directions.py:213-256) on the CPU.
    Returns (adjusted dirs or None, final ridge, unadjusted main dirs).  A
    dict passed as `stages` receives the ridge after the hysteresis, before
    the cleaning ("ridge_hysteresis")."""
    qeigs = np.require(qeigs, np.float32, ["C", "A"])
    response = np.require(response, np.float32, ["C", "A"])
    voxel_size = tuple(np.multiply(np.ones(3), voxel_size))
    try:
        len(threshold)
        threshold = tuple(sorted(threshold))
        hyst, lower = True, threshold[0]
    except TypeError:
        hyst, lower = False, threshold
    ridge = O.detect_ridges(response, qeigs, lower)
    if hyst:
        sure = np.logical_and(ridge, response >= threshold[1])
        ridge[:] = hysteresis_threshold(ridge, sure)
    if stages is not None:
        stages["ridge_hysteresis"] = ridge.copy()
    adjusted = None
    main = None
    if (not ridge_detection_only) or clean:
        main = O.extract_main_directions(qeigs)
        coords, rdirs = adjust_ridge_directions(ridge, main, voxel_size)
        if clean:
            ridge = clean_ridge(ridge, coords, rdirs, voxel_size)
            if not ridge_detection_only:
                coords, rdirs = adjust_ridge_directions(ridge, main, voxel_size)
        if not ridge_detection_only:
            adjusted = O.adjust_nonridge_signs(main, coords, rdirs, voxel_size)
    return adjusted, ridge, main
