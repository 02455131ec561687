"""Parity of the CUDA Frangi stage (csrc/frangi.cu) with the oracle.

Tolerances (fp32 with fused multiply-adds and the hardware rsqrt against the
reference's sequential double-promoted arithmetic):
  Hessian entries within 2e-5 of the scale's max |H|;
  eigenvalues within 1e-5 of float64 eigvalsh relative to the matrix's max |lambda|;
  eigenvector rotation reproducing H within 1e-4 of max |H|;
  vesselness within 1e-4 absolute; the quaternion of the maximising scale the
  same as the oracle's (as a rotation) wherever the best two scales' responses
  differ by more than 1e-3.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import inputs as I  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


def _sym(h):
    h = h.reshape(-1, 6)
    return np.stack([h[:, 0], h[:, 3], h[:, 4], h[:, 3], h[:, 1], h[:, 5], h[:, 4], h[:, 5], h[:, 2]],
                    -1).reshape(-1, 3, 3).astype(np.float64)


def _rot(sq):
    phi, th, psi = [sq[..., k].astype(np.float64) for k in range(3)]
    w = np.cos((phi + psi) / 2) * np.cos(th / 2)
    x = np.cos((phi - psi) / 2) * np.sin(th / 2)
    y = np.sin((phi - psi) / 2) * np.sin(th / 2)
    z = np.sin((phi + psi) / 2) * np.cos(th / 2)
    return np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                     2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                     2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1).reshape(-1, 3, 3)


# radius round(4 sigma): 4.4 gives 18, beyond the passes instantiated per
# radius (1-16), so the last case runs the kernels for any radius
@pytest.mark.parametrize("shape,sigma", [((20, 24, 28), (1.0, 1.0, 1.0)), ((33, 17, 40), (3.0, 2.0, 2.5)),
                                         ((5, 70, 9), (1.5, 1.5, 1.5)), ((1, 12, 13), (1.0, 1.0, 1.0)),
                                         ((24, 20, 40), (4.4, 4.4, 4.4))])
def test_hessian_matches_oracle(shape, sigma):
    from miccai2016_gb300.qfrangi_gpu import hessian
    rng = np.random.RandomState(sum(shape))
    img = rng.normal(0.5, 0.5, shape).astype(np.float32)
    h = hessian(img, sigma)
    r = O.hessian(img, sigma)
    assert h.shape == shape + (6,)
    assert np.max(np.abs(h - r)) <= 2e-5 * max(1e-12, float(np.max(np.abs(r))))


def test_eigs_against_float64_and_reconstruction():
    from miccai2016_gb300.qfrangi_gpu import eigendecomposition
    rng = np.random.RandomState(3)
    h = rng.normal(size=(200000, 6)).astype(np.float32)
    h[:1000] *= 1e-12
    h[1000:2000, 3:] = 0
    h[2000:3000, :3] = 1.0
    e = eigendecomposition(h)
    ev = np.linalg.eigvalsh(_sym(h))
    ev = np.take_along_axis(ev, np.argsort(np.abs(ev), 1), 1)
    mx = np.maximum(np.abs(ev).max(1, keepdims=True), 1e-300)
    assert np.max(np.abs(e[:, :3] - ev) / mx) <= 1e-5
    R = _rot(e[:, 3:])
    rec = R @ (e[:, :3, None].astype(np.float64) * np.transpose(R, (0, 2, 1)))
    H = _sym(h)
    scale = np.abs(H).reshape(len(H), -1).max(1)[:, None, None]
    assert np.max(np.abs(rec - H) / np.maximum(scale, 1e-300)) <= 1e-4


def test_eigs_nan_in_nan_out():
    from miccai2016_gb300.qfrangi_gpu import eigendecomposition
    e = eigendecomposition(np.full((4, 6), np.nan, np.float32))
    assert np.all(np.isnan(e))


@pytest.mark.parametrize("name", I.FRANGI_CASES)
def test_frangi_matches_golden(name):
    from miccai2016_gb300.qfrangi_gpu import FeatureFilter, VesselnessCalculation
    img, kw = I.frangi_case(name)
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    p = VesselnessCalculation.Parameters()
    p.alpha, p.beta, p.c, p.bright_objects, p.scales = kw["alpha"], kw["beta"], kw["c"], kw["bright"], kw["scales"]
    ff = FeatureFilter(p)
    val, quat, slc = ff.execute_for(img, None, kw["voxel_size"])
    assert slc is None and val.shape == img.shape and quat.shape == img.shape + (3,)
    np.testing.assert_allclose(ff.last_c, g["c"], rtol=1e-4)
    assert np.max(np.abs(val - g["val"])) <= 1e-4
    _check_quats(img, kw, val, quat, g["val"], g["quat"])


def _check_quats(img, kw, val, quat, rval, rquat):
    # per-scale responses of the oracle to find voxels with a clear winner
    sig = O.frangi_scales(kw["scales"], np.ones(3) if kw["voxel_size"] is None else kw["voxel_size"])
    vs = []
    for s in sig:
        e = O.eigs(O.hessian(img, s))
        v = np.full(img.shape, -np.inf, np.float32)
        q = np.zeros(img.shape + (3,), np.float32)
        c = kw["c"] if kw["c"] is not None else 0.5 * O.lib().oracle_max_norm(e.size // 6, O._ptr(e))
        O.lib().oracle_update_vesselness(v.size, O._ptr(v), O._ptr(q), O._ptr(e), kw["alpha"], kw["beta"], c,
                                         int(kw["bright"]))
        vs.append(v)
    vs = np.sort(np.stack(vs), axis=0)
    clear = (vs[-1] - (vs[-2] if len(vs) > 1 else -np.inf)) > 1e-3
    clear &= np.isfinite(rval) & (rval > 1e-3)
    Ra = _rot(quat.reshape(-1, 3))[clear.ravel()]
    Rb = _rot(rquat.reshape(-1, 3))[clear.ravel()]
    # columns are eigenvectors up to sign
    dots = np.abs(np.einsum("nij,nij->nj", Ra, Rb))
    assert dots.size == 0 or np.min(dots) > 1 - 1e-3


def test_frangi_helix_phantom_bright_and_roi():
    from miccai2016_gb300 import phantom as P
    from miccai2016_gb300.qfrangi_gpu import FeatureFilter, VesselnessCalculation
    cfg = P.CONFIG_PLAIN_64
    noisy, truth = P.helix_phantom(cfg["shape"], cfg["tube_radius"], cfg["helix_radius"], cfg["pitch"],
                                   cfg["sigma"], cfg["seed"])
    p = VesselnessCalculation.Parameters()
    p.bright_objects, p.scales = True, (1, 3, 3)
    val, quat, _ = FeatureFilter(p).execute_for(noisy, None, (1, 1, 1))
    rval, rquat, rc = O.frangi(noisy, (1, 3, 3))
    assert np.max(np.abs(val - rval)) <= 1e-4
    # a region of interest crops with the largest kernel arm as margin
    roi = np.zeros(noisy.shape, bool)
    roi[20:30, 25:35, 30:40] = True
    v2, q2, slc = FeatureFilter(p).execute_for(noisy, roi, (1, 1, 1))
    assert slc == (slice(8, 42, 1), slice(13, 47, 1), slice(18, 52, 1))
    assert v2.shape == (34, 34, 34)
