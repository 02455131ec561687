"""26-connected labelling on the GPU (m16_label26) against
scipy.ndimage.label with a 3 x 3 x 3 structure of ones: the same labels and
count on sparse, dense, percolating and empty masks and thin volumes; the
hysteresis and the adjuster with GPU labels against the reference logic."""
import contextlib
import io

import numpy as np
import pytest
import scipy.ndimage

from oracle import adjust as A

pytestmark = pytest.mark.gpu


def _scipy(mask):
    lab, n = scipy.ndimage.label(mask, structure=np.ones((3, 3, 3), int))
    return lab, n


@pytest.mark.parametrize("shape", [(40, 33, 50), (1, 64, 64), (7, 1, 300), (1, 1, 1), (96, 96, 96)])
@pytest.mark.parametrize("density", [0.0, 0.05, 0.25, 0.45, 1.0])
def test_labels_equal_scipy(shape, density):
    from miccai2016_gb300.labeling import label26
    rng = np.random.RandomState(int(density * 100) + sum(shape))
    mask = rng.uniform(size=shape) < density
    lab, n = label26(mask)
    ref, rn = _scipy(mask)
    assert n == rn
    assert np.array_equal(lab, ref)


def test_long_thin_components_and_diagonals():
    from miccai2016_gb300.labeling import label26
    mask = np.zeros((30, 40, 50), bool)
    for k in range(28):                    # a diagonal staircase: connected only through corners
        mask[k, k, k] = True
    mask[:, 20, 45] = True                 # a full-length line
    mask[5, 30:, ::2] = True               # separate dots, one component each
    lab, n = label26(mask)
    ref, rn = _scipy(mask)
    assert n == rn and np.array_equal(lab, ref)


def test_hysteresis_with_gpu_labels_equals_the_flood_fill():
    from miccai2016_gb300.ridge_detection import hysteresis_threshold
    rng = np.random.RandomState(2)
    for p in (0.1, 0.3):
        cand = rng.uniform(size=(20, 22, 24)) < p
        sure = np.logical_and(cand, rng.uniform(size=cand.shape) < 0.05)
        a = A.hysteresis_threshold(cand.copy(), sure.copy())
        b = hysteresis_threshold(cand.copy(), sure.copy(), labeler="gpu")
        assert np.array_equal(a, b)


def test_adjuster_with_gpu_labels_and_tree_matches_the_reference_logic():
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
    assert obj.labeler == "gpu" and obj.mst_local == "gpu"
    c1, d1 = A.adjust_ridge_directions(ridge, main, (1.0, 1.0, 1.0))
    c2, d2 = obj._adjust_ridge_directions(ridge, main)
    with contextlib.redirect_stdout(io.StringIO()):
        k1 = A.clean_ridge(ridge, c1, d1, (1.0, 1.0, 1.0))
        k2 = obj._do_clean_ridge(ridge, c2, d2)
    assert np.array_equal(k1, k2)
