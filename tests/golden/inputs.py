"""
Seeded inputs of the golden fixtures.  numpy's RandomState stream is the same
on every platform, so the fixtures store only outputs; the inputs are rebuilt
from these functions (tests/golden/make_golden.py writes the outputs).
"""
from __future__ import annotations

import numpy as np


def random_squeezed(rng, shape):
    """Squeezed quaternions (phi, theta, psi) with uniform angles."""
    return np.stack([rng.uniform(-np.pi, np.pi, shape), rng.uniform(0, np.pi, shape),
                     rng.uniform(-np.pi, np.pi, shape)], -1).astype(np.float32)


def maxflow_case(name):
    """(inputs dict, solver kwargs) of one max-flow fixture."""
    if name == "mf_const_unsup":
        rng = np.random.RandomState(11)
        shape = (20, 24, 28)
        eigs = (1.0, 10 ** -1.5, 10 ** -1.5)
        labels = None
        scaling = (1, 1, 1)
        kw = dict(num_iter=60, update=10, error_bound=-1.0)
    elif name == "mf_point_sup":
        rng = np.random.RandomState(12)
        shape = (17, 10, 33)
        eigs = None
        labels = "random"
        scaling = (1.5, 0.7, 1.2)
        kw = dict(num_iter=45, update=7, error_bound=-1.0)
    elif name == "mf_stop":
        rng = np.random.RandomState(13)
        shape = (16, 16, 16)
        eigs = (1.0, 1.0, 1.0)
        labels = None
        scaling = (1, 1, 1)
        kw = dict(num_iter=400, update=5, error_bound=2e-3)
    else:
        raise KeyError(name)
    img = rng.normal(0.5, 0.5, shape).astype(np.float32)
    quats = random_squeezed(rng, shape)
    alpha = rng.uniform(0.01, 0.5, shape).astype(np.float32)
    cs = rng.uniform(0, 1, shape).astype(np.float32)
    ct = rng.uniform(0, 1, shape).astype(np.float32)
    if eigs is None:
        eigs = rng.uniform(0.01, 2.0, shape + (3,))
    if labels == "random":
        labels = rng.randint(0, 3, shape).astype(np.uint8)
    inputs = dict(img=img, quats=quats, eigs=eigs, alpha=alpha, cs=cs, ct=ct, labels=labels, scaling=scaling)
    return inputs, kw


MAXFLOW_CASES = ("mf_const_unsup", "mf_point_sup", "mf_stop")


def gvf_case(name):
    """(vfield, kwargs) of one GVF fixture."""
    if name == "gvf_basic":
        rng = np.random.RandomState(21)
        shape = (12, 10, 14)
        kw = dict(mu=0.2, maxiter=40, update=7, tol=0.0, normalize=False, voxel_size=None)
    elif name == "gvf_aniso_norm":
        rng = np.random.RandomState(22)
        shape = (9, 13, 6)
        kw = dict(mu=10 ** 0.5, maxiter=30, update=10, tol=0.0, normalize=True, voxel_size=(1.5, 0.8, 1.1))
    elif name == "gvf_tol":
        rng = np.random.RandomState(23)
        shape = (10, 10, 10)
        kw = dict(mu=0.2, maxiter=200, update=5, tol=2e-3, normalize=False, voxel_size=None)
    else:
        raise KeyError(name)
    return unit_field(rng, shape), kw


def unit_field(rng, shape):
    """Random directions scaled by uniform [0, 1) magnitudes, like the
    vesselness-weighted direction fields GVF diffuses (|v| <= 1 keeps the
    explicit scheme stable)."""
    d = rng.normal(size=shape + (3,))
    d /= np.maximum(np.linalg.norm(d, axis=-1, keepdims=True), 1e-12)
    return (d * rng.uniform(0, 1, shape)[..., None]).astype(np.float32)


GVF_CASES = ("gvf_basic", "gvf_aniso_norm", "gvf_tol")


def frangi_case(name):
    """(image, kwargs of oracle.frangi) of one Frangi fixture."""
    if name == "frangi_bright":
        rng = np.random.RandomState(31)
        shape = (10, 12, 11)
        kw = dict(scales=(1, 3, 3), voxel_size=None, alpha=0.5, beta=0.5, c=None, bright=True)
    elif name == "frangi_dark_aniso":
        rng = np.random.RandomState(32)
        shape = (11, 9, 20)
        kw = dict(scales=(1.0, 2.0, 2), voxel_size=(1.5, 1.0, 0.8), alpha=0.5, beta=0.5, c=0.25, bright=False)
    else:
        raise KeyError(name)
    img = rng.normal(0.5, 0.5, shape).astype(np.float32)
    return img, kw


FRANGI_CASES = ("frangi_bright", "frangi_dark_aniso")


def directions_case():
    """Inputs of the direction-kernel fixture: response, squeezed quaternions,
    vectors (with a zero vector), a ridge list with duplicate distances."""
    rng = np.random.RandomState(41)
    shape = (11, 14, 9)
    resp = rng.uniform(0, 1, shape).astype(np.float32)
    quats = random_squeezed(rng, shape)
    vecs = rng.normal(size=shape + (3,)).astype(np.float32)
    vecs[0, 0, 0] = 0.0
    vecs[1, 2, 3] = (0.0, 0.0, 1.0)
    R = 29
    coords = np.stack([rng.randint(0, s, R) for s in shape], -1).astype(np.uint16)
    coords[5] = coords[4] + np.array([2, 0, 0], np.uint16) if coords[4][0] + 2 < shape[0] else coords[5]
    rdirs = rng.normal(size=(R, 3)).astype(np.float32)
    return dict(resp=resp, quats=quats, vecs=vecs, coords=coords, rdirs=rdirs)
