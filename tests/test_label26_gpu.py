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


@pytest.mark.parametrize("shape", [(40, 33, 50), (1, 64, 64), (7, 1, 300), (1, 1, 1)])
@pytest.mark.parametrize("density", [0.0, 0.2, 0.5, 1.0])
def test_six_connected_labels_equal_scipys_default(shape, density):
    from miccai2016_gb300.labeling import label
    rng = np.random.RandomState(int(density * 100) + sum(shape) + 6)
    mask = rng.uniform(size=shape) < density
    lab, n = label(mask, connectivity=6)
    ref, rn = scipy.ndimage.label(mask)
    assert n == rn and np.array_equal(lab, ref)


def _blobs(rng, shape, k):
    seg = np.zeros(shape, np.float32)
    for _ in range(k):
        c = rng.randint(0, shape, 3)
        r = rng.randint(1, 5, 3)
        sl = tuple(slice(max(0, c[a] - r[a]), c[a] + r[a]) for a in range(3))
        seg[sl] = rng.uniform(0.5, 1.0)
    return seg + rng.uniform(0, 0.49, shape).astype(np.float32)


@pytest.mark.parametrize("seed", range(6))
def test_dice_of_the_largest_component_equals_the_host(seed):
    from miccai2016_gb300 import phantom as P
    from miccai2016_gb300.labeling import dice_largest
    rng = np.random.RandomState(seed)
    shape = tuple(rng.randint(8, 48, 3))
    seg = _blobs(rng, shape, rng.randint(1, 12))
    truth = _blobs(rng, shape, 3) >= 0.5
    if seed == 4:
        seg[3, 3, 3] = np.nan               # NaN is background, as numpy's comparison
    assert dice_largest(seg, truth) == P.dice_largest(seg, truth)


def test_dice_largest_ties_empty_and_full():
    from miccai2016_gb300 import phantom as P
    from miccai2016_gb300.labeling import dice_largest
    shape = (10, 12, 14)
    seg = np.zeros(shape, np.float32)
    seg[1:3, 1:3, 1:3] = 1                  # two components of equal size: the first label wins
    seg[6:8, 6:8, 6:8] = 1
    truth = np.zeros(shape, bool)
    truth[6:8, 6:8, 6:8] = True
    assert dice_largest(seg, truth) == P.dice_largest(seg, truth) == 0.0
    truth[1:3, 1:3, 1:2] = True
    assert dice_largest(seg, truth) == P.dice_largest(seg, truth)
    assert dice_largest(np.zeros(shape, np.float32), truth) == 0.0
    full = np.ones(shape, np.float32)
    assert dice_largest(full, truth) == P.dice_largest(full, truth)
