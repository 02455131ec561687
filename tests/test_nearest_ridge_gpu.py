"""The indexed nearest-ridge sign flip (m16_adjust_nonridge_signs_indexed)
against the brute-force kernel (m16_adjust_nonridge_signs) and the oracle
(adjustNonRidgeSigns, src/clcode/adjust_directions.cl:182-246): bit-exact
outputs on dense, sparse, clustered, duplicated, tied and out-of-volume ridge
lists, thin volumes and anisotropic voxel sizes."""
import ctypes
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import inputs as I  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _run(vecs, coords, rdirs, scaling, indexed):
    import torch
    from miccai2016_gb300 import _native as N
    L = N.lib()
    d = torch.from_numpy(np.ascontiguousarray(vecs, np.float32)).cuda()
    c = torch.from_numpy(np.ascontiguousarray(coords, np.uint16).view(np.int16)).cuda()
    r = torch.from_numpy(np.ascontiguousarray(rdirs, np.float32)).cuda()
    sc = (ctypes.c_double * 3)(*scaling)
    d0, d1, d2 = vecs.shape[:3]
    if indexed:
        ws = N.workspace(L.m16_adjust_nonridge_signs_workspace_bytes(d0, d1, d2, len(coords)))
        st = L.m16_adjust_nonridge_signs_indexed(N.ptr(d), d0, d1, d2, N.ptr(c), N.ptr(r), len(coords), sc,
                                                 N.ptr(ws), ws.numel(), N.stream_ptr())
    else:
        st = L.m16_adjust_nonridge_signs(N.ptr(d), d0, d1, d2, N.ptr(c), N.ptr(r), len(coords), sc, N.stream_ptr())
    N.check("sign flip", st)
    return d.cpu().numpy()


def _check(vecs, coords, rdirs, scaling, oracle=True):
    a = _run(vecs, coords, rdirs, scaling, indexed=True)
    b = _run(vecs, coords, rdirs, scaling, indexed=False)
    assert np.array_equal(_bits(a), _bits(b))
    if oracle:
        assert np.array_equal(_bits(a), _bits(O.adjust_nonridge_signs(vecs, coords, rdirs, scaling)))
    return a


SCALINGS = [(1, 1, 1), (1.5, 0.7, 1.2), (0.1, 10.0, 1.0), (0.3333, 0.3333, 0.3333)]


@pytest.mark.parametrize("density", [0.3, 0.02, 1e-4])
@pytest.mark.parametrize("scaling", SCALINGS)
def test_random_ridge_lists(density, scaling):
    shape = (40, 33, 50)
    rng = np.random.RandomState(int(density * 1e4) + 7)
    v = rng.normal(size=shape + (3,)).astype(np.float32)
    R = max(1, int(density * np.prod(shape)))
    coords = np.stack([rng.randint(0, s, R) for s in shape], -1).astype(np.uint16)
    rd = rng.normal(size=(R, 3)).astype(np.float32)
    _check(v, coords, rd, scaling)


@pytest.mark.parametrize("scaling", SCALINGS[:2])
def test_clustered_points_and_far_voxels(scaling):
    shape = (48, 40, 44)
    rng = np.random.RandomState(3)
    v = rng.normal(size=shape + (3,)).astype(np.float32)
    R = 500
    coords = np.stack([rng.randint(0, 5, R), rng.randint(0, 6, R), rng.randint(0, 4, R)], -1).astype(np.uint16)
    rd = rng.normal(size=(R, 3)).astype(np.float32)
    _check(v, coords, rd, scaling)


def test_duplicates_and_ties_go_to_the_lowest_index():
    shape = (9, 9, 9)
    rng = np.random.RandomState(5)
    v = rng.normal(size=shape + (3,)).astype(np.float32)
    # a lattice with spacing 2 (many voxels equidistant from several points),
    # points listed up to three times with different directions
    g = np.stack(np.meshgrid(*[np.arange(0, 9, 2)] * 3, indexing="ij"), -1).reshape(-1, 3)
    coords = np.concatenate([g[::-1], g, g[::3]]).astype(np.uint16)
    rd = rng.normal(size=(len(coords), 3)).astype(np.float32)
    for sc in [(1, 1, 1), (2, 2, 2), (1, 2, 1)]:
        _check(v, coords, rd, sc)


def test_coordinates_beyond_the_volume():
    shape = (12, 10, 14)
    rng = np.random.RandomState(11)
    v = rng.normal(size=shape + (3,)).astype(np.float32)
    R = 60
    coords = np.stack([rng.randint(0, s + 9, R) for s in shape], -1).astype(np.uint16)
    rd = rng.normal(size=(R, 3)).astype(np.float32)
    for sc in SCALINGS[:2]:
        _check(v, coords, rd, sc)


@pytest.mark.parametrize("shape,R", [((1, 20, 20), 7), ((7, 64, 3), 40), ((1, 1, 1), 1), ((2, 1, 300), 3),
                                     ((130, 3, 5), 25)])
def test_thin_volumes(shape, R):
    rng = np.random.RandomState(R)
    v = rng.normal(size=shape + (3,)).astype(np.float32)
    coords = np.stack([rng.randint(0, s, R) for s in shape], -1).astype(np.uint16)
    rd = rng.normal(size=(R, 3)).astype(np.float32)
    for sc in SCALINGS[:3]:
        _check(v, coords, rd, sc)


def test_golden_fixture_through_the_index():
    d = I.directions_case()
    g = np.load(os.path.join(HERE, "golden", "directions.npz"))
    assert np.array_equal(_bits(_run(d["vecs"], d["coords"], d["rdirs"], (1, 1, 1), True)), _bits(g["adjust_iso"]))
    assert np.array_equal(_bits(_run(d["vecs"], d["coords"], d["rdirs"], (1.5, 0.7, 1.2), True)),
                          _bits(g["adjust_aniso"]))


def test_large_volume_matches_brute_force():
    # 96^3 with a helix-like dense ridge band plus scattered points
    shape = (96, 96, 96)
    rng = np.random.RandomState(17)
    v = rng.normal(size=shape + (3,)).astype(np.float32)
    t = np.linspace(0, 6 * np.pi, 4000)
    band = np.stack([8 + t * 12, 48 + 30 * np.sin(t), 48 + 30 * np.cos(t)], -1)
    band = np.clip(np.round(band + rng.normal(scale=1.5, size=band.shape)), 0, 95)
    scatter = np.stack([rng.randint(0, 96, 3000) for _ in range(3)], -1)
    coords = np.concatenate([band, scatter]).astype(np.uint16)
    rd = rng.normal(size=(len(coords), 3)).astype(np.float32)
    _check(v, coords, rd, (1, 1, 1), oracle=False)
    _check(v, coords, rd, (0.8, 1.1, 1.0), oracle=False)
