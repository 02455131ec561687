"""The Frangi oracle (oracle/frangi.c) against golden fixtures made from the
reference's convolve_naive.cl, qeigs.cl and frangi.cl, live against those
kernels where the reference checkout exists, and the Jacobi eigenvalues
against float64 numpy.linalg.eigvalsh."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from oracle import oracle as O  # noqa: E402
import inputs as I  # noqa: E402


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("name", I.FRANGI_CASES)
def test_oracle_matches_golden(name):
    img, kw = I.frangi_case(name)
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    val, quat, c = O.frangi(img, **kw)
    assert np.array_equal(_bits(val), _bits(g["val"]))
    assert np.array_equal(_bits(quat), _bits(g["quat"]))
    assert np.array_equal(c, g["c"])
    sig = O.frangi_scales(kw["scales"], np.ones(3) if kw["voxel_size"] is None else kw["voxel_size"])
    for k, s in enumerate(sig[:len(g["hessian"])]):
        h = O.hessian(img, s)
        assert np.array_equal(_bits(h), _bits(g["hessian"][k]))
        assert np.array_equal(_bits(O.eigs(h)), _bits(g["eigs"][k]))


def _sym(h):
    return np.stack([h[..., 0], h[..., 3], h[..., 4], h[..., 3], h[..., 1], h[..., 5], h[..., 4], h[..., 5],
                     h[..., 2]], -1).reshape(-1, 3, 3).astype(np.float64)


def test_jacobi_eigenvalues_against_float64():
    rng = np.random.RandomState(5)
    h = rng.normal(size=(20000, 6)).astype(np.float32)
    h[:100] *= 1e-12          # small (the reference's float Jacobi underflows to NaN below ~1e-19)
    h[100:200, 3:] = 0        # already diagonal
    h[200:300, :3] = 1.0      # degenerate diagonal
    e = O.eigs(h)
    ev = np.linalg.eigvalsh(_sym(h))
    ev = np.take_along_axis(ev, np.argsort(np.abs(ev), 1), 1)
    mx = np.maximum(np.abs(ev).max(1, keepdims=True), 1e-300)
    assert np.max(np.abs(e[:, :3] - ev) / mx) <= 1e-5


def test_jacobi_rotation_reconstructs_the_matrix():
    rng = np.random.RandomState(6)
    h = rng.normal(size=(2000, 6)).astype(np.float32)
    e = O.eigs(h)
    # expand the squeezed quaternion (z-x-z Euler) to R, check R diag(l) R^T = H
    phi, th, psi = e[:, 3].astype(np.float64), e[:, 4].astype(np.float64), e[:, 5].astype(np.float64)
    w = np.cos((phi + psi) / 2) * np.cos(th / 2)
    x = np.cos((phi - psi) / 2) * np.sin(th / 2)
    y = np.sin((phi - psi) / 2) * np.sin(th / 2)
    z = np.sin((phi + psi) / 2) * np.cos(th / 2)
    R = np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                  2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                  2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1).reshape(-1, 3, 3)
    rec = R @ (e[:, :3, None].astype(np.float64) * np.transpose(R, (0, 2, 1)))
    H = _sym(h)
    assert np.max(np.abs(rec - H)) / np.max(np.abs(H)) < 1e-5


def test_nan_matrix_gives_nan():
    h = np.full((1, 6), np.nan, np.float32)
    assert np.all(np.isnan(O.eigs(h)))


def test_underflowing_matrix_gives_nan_like_the_reference():
    # squares of ~1e-30 entries underflow in float, rsqrt(0) -> inf, c * inf -> NaN:
    # the reference's qeigs.cl returns NaN for such matrices and so does the oracle
    h = (np.random.RandomState(1).normal(size=(4, 6)) * 1e-30).astype(np.float32)
    assert np.all(np.isnan(O.eigs(h)))


@pytest.mark.parametrize("shape", [(5, 7, 9), (2, 3, 4), (12, 6, 8)])
def test_oracle_matches_reference_kernels(has_ref, shape):
    if not has_ref:
        pytest.skip("reference checkout not present")
    rng = np.random.RandomState(sum(shape))
    img = rng.normal(0.5, 0.5, shape).astype(np.float32)
    for kw in [dict(scales=(1, 3, 3)), dict(scales=(0.8, 1.6, 2), voxel_size=(1.2, 0.9, 1.0), bright=False)]:
        a = O.frangi(img, **kw)
        b = O.ref_frangi(img, **kw)
        assert np.array_equal(_bits(a[0]), _bits(b[0]))
        assert np.array_equal(_bits(a[1]), _bits(b[1]))


def test_taps_match_formula():
    for s in (0.7, 1.0, 2.5, 7.2):
        t0 = O.gauss_taps(s, 0)
        assert len(t0) == 2 * int(4 * s + 0.5) + 1
        assert abs(float(np.sum(t0.astype(np.float64))) - 1.0) < 1e-6
        t1 = O.gauss_taps(s, 1)
        assert np.allclose(t1, -t1[::-1])
