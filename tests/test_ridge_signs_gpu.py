"""The sign propagation on the device (csrc/ridge_forest.cu through
ridge_mst.propagate_signs_device): bit for bit the reference's
point-by-point loop (adjust_directions.py:382-415) and the host propagation,
on trees and forests with zero, near-zero (np.dot decides) and NaN dot
products, long chains, and invalid input rejected."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from test_ridge_host import _loop  # noqa: E402

pytestmark = pytest.mark.gpu


def _forest(rng, n, drop=0.05, chain=False):
    if chain:   # long paths, as ridge trees are
        par = np.maximum(0, np.arange(n) - rng.randint(1, 4, n))
    else:
        par = np.array([rng.randint(0, i) if i else 0 for i in range(n)])
    keep = rng.uniform(size=n) > drop
    a = np.arange(1, n)[keep[1:]]
    b = par[1:][keep[1:]]
    perm = rng.permutation(n)
    return perm[a].astype(np.int64), perm[b].astype(np.int64)


def _device(a, b, dirs):
    import torch
    from miccai2016_gb300.ridge_mst import propagate_signs_device
    return propagate_signs_device(torch.from_numpy(dirs).cuda(), a, b).cpu().numpy()


def _near_zero_dots(rng, a, b, dirs, count):
    # edges whose dot lies within float32 rounding of zero: np.dot decides
    k = rng.randint(0, len(a), count)
    dirs[a[k]] = np.float32([1, 1, 0])
    dirs[b[k]] = np.float32([1, -(1 - 2.0 ** -22), 0])


@pytest.mark.parametrize("seed", range(12))
def test_device_propagation_equals_the_loop(seed):
    rng = np.random.RandomState(100 + seed)
    n = int(rng.choice([1, 2, 10, 700, 5000]))
    a, b = _forest(rng, n)
    dirs = rng.normal(size=(n, 3)).astype(np.float32)
    if n > 6:
        dirs[rng.randint(0, n, n // 20 + 1)] = 0.0                     # zero dots
        dirs[1], dirs[2], dirs[3] = [1, 0, 0], [0, 1, 0], [1e-8, 1, 0]  # exact and near-zero
        if seed % 3 == 0:
            dirs[4] = [np.nan, 0, 1]
        if len(a):
            _near_zero_dots(rng, a, b, dirs, 3)
    x = _loop(n, a, b, dirs)
    y = _device(a, b, dirs)
    assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


@pytest.mark.parametrize("chain", [False, True])
def test_device_propagation_equals_the_host_on_large_forests(chain):
    from miccai2016_gb300.ridge_mst import propagate_signs
    rng = np.random.RandomState(7 + chain)
    n = 300_000
    a, b = _forest(rng, n, drop=0.001, chain=chain)
    dirs = rng.normal(size=(n, 3)).astype(np.float32)
    dirs[rng.randint(0, n, 300)] = 0.0
    dirs[rng.randint(0, n, 30)] = np.nan
    _near_zero_dots(rng, a, b, dirs, 200)
    x = propagate_signs(n, a, b, dirs)
    y = _device(a, b, dirs)
    assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_invalid_codes_and_edges_are_rejected():
    import torch
    from miccai2016_gb300 import _native as N
    L = N.lib()
    n = 5
    a = torch.tensor([1, 2, 3], dtype=torch.int32, device="cuda")
    b = torch.tensor([0, 1, 2], dtype=torch.int32, device="cuda")
    signs = torch.empty(n, dtype=torch.int8, device="cuda")
    ws = N.workspace(L.m16_ridge_signs_workspace_bytes(n, 3))
    for bad in ([1, 3, 1], [1, 4, -1], [7, 1, 1]):
        codes = torch.tensor(bad, dtype=torch.int8, device="cuda")
        st = L.m16_ridge_signs(n, N.ptr(a), N.ptr(b), N.ptr(codes), 3, N.ptr(signs), N.ptr(ws), ws.numel(),
                               N.stream_ptr())
        assert st == 2   # M16_ERR_BAD_ARG
    # an endpoint outside [0, n): code 4, then rejected
    dirs = torch.ones((n, 3), dtype=torch.float32, device="cuda")
    b2 = torch.tensor([0, 9, 2], dtype=torch.int32, device="cuda")
    codes = torch.empty(3, dtype=torch.int8, device="cuda")
    assert L.m16_ridge_edge_codes(N.ptr(dirs), n, N.ptr(a), N.ptr(b2), 3, N.ptr(codes), N.stream_ptr()) == 0
    assert codes.cpu().tolist() == [1, 4, 1]
    st = L.m16_ridge_signs(n, N.ptr(a), N.ptr(b2), N.ptr(codes), 3, N.ptr(signs), N.ptr(ws), ws.numel(),
                           N.stream_ptr())
    assert st == 2
    assert L.m16_ridge_signs_workspace_bytes(n, n) == 0   # a forest has fewer edges than points
