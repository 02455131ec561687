"""m16_segment_direction_sums (csrc/host_sums.cpp), the per-segment summed
directions of the ridge cleaning (adjust_directions.py:319-337), against
np.bincount with the reference's float64 products as weights: bit for bit.

The library's host code is built with multiply-add contraction off, so that
the products are rounded before they are added on every host; the same check
runs once more among the GPU tests, which run on the Arm GPU hosts."""
import ctypes

import numpy as np
import pytest


def _sums(L, labels, dirs, vs, n_lab):
    out = np.empty((n_lab, 3), np.float64)
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    pl = np.ascontiguousarray(labels, np.int32)
    d = np.ascontiguousarray(dirs, np.float32)
    v = np.ascontiguousarray(vs, np.float64)
    st = L.m16_segment_direction_sums(vp(pl), vp(d), len(pl), vp(v), n_lab, vp(out))
    return st, out


def _check_against_bincount():
    from miccai2016_gb300 import _native as N
    L = N.lib()
    rng = np.random.RandomState(319)
    for n, n_lab, vs in ((200_000, 7, (1, 1, 1)), (150_000, 3000, (0.7, 1.3, 2.1)), (50_000, 50_000, (1e-3, 1, 7.5)),
                         (1, 1, (1, 1, 1)), (0, 4, (2.0, 0.5, 1.0))):
        labels = np.sort(rng.randint(0, n_lab, n)) if n_lab < n else rng.randint(0, n_lab, n)
        dirs = rng.normal(size=(n, 3)).astype(np.float32)
        dirs[::97] *= np.float32(1e-20)
        dirs[1::89] *= np.float32(3e7)
        st, out = _sums(L, labels, dirs, vs, n_lab)
        assert st == 0
        scaled = dirs * tuple(vs)   # float32 * tuple -> float64 products, as the reference forms them
        want = np.stack([np.bincount(labels, weights=scaled[:, k], minlength=n_lab) for k in range(3)], -1)
        assert np.array_equal(out.view(np.uint64), want.view(np.uint64)), (n, n_lab, vs)
    # a label outside 0 .. num_labels - 1
    st, _ = _sums(L, np.array([0, 5], np.int32), np.ones((2, 3), np.float32), (1, 1, 1), 5)
    assert st == N.M16_ERR_BAD_ARG


def test_segment_sums_equal_bincount():
    _check_against_bincount()


@pytest.mark.gpu
def test_segment_sums_equal_bincount_on_the_gpu_host():
    _check_against_bincount()
