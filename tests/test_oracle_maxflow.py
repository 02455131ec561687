"""The max-flow oracle (oracle/maxflow.c) against the golden fixtures made
from the reference's own kernels, and live against those kernels where the
reference checkout is present.  CPU only."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from oracle import oracle as O  # noqa: E402
import inputs as I  # noqa: E402


def _bits_equal(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


@pytest.mark.parametrize("name", I.MAXFLOW_CASES)
def test_oracle_matches_golden(name):
    inp, kw = I.maxflow_case(name)
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    u, iters, resid = O.maxflow_solve(inp["img"], inp["quats"], inp["eigs"], inp["alpha"], inp["cs"], inp["ct"],
                                      labels=inp["labels"], scaling=inp["scaling"], **kw)
    assert iters == int(g["iterations"])
    assert _bits_equal(u, g["u"])
    np.testing.assert_allclose(resid, g["residuals"], rtol=1e-6, atol=0)


def test_golden_stop_case_stops_early():
    g = np.load(os.path.join(HERE, "golden", "mf_stop.npz"))
    inp, kw = I.maxflow_case("mf_stop")
    assert int(g["iterations"]) < kw["num_iter"]
    assert g["residuals"][-1] < kw["error_bound"] <= g["residuals"][-2]


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 5, 1), (2, 3, 4), (5, 7, 9), (3, 1, 8)])
@pytest.mark.parametrize("supervised", [False, True])
@pytest.mark.parametrize("pointwise", [False, True])
def test_oracle_matches_reference_kernels(has_ref, shape, supervised, pointwise):
    if not has_ref:
        pytest.skip("reference checkout not present")
    rng = np.random.RandomState(hash((shape, supervised, pointwise)) % 2 ** 31)
    img = rng.normal(0.5, 0.5, shape).astype(np.float32)
    q = I.random_squeezed(rng, shape)
    alpha = rng.uniform(0.01, 0.5, shape).astype(np.float32)
    cs = rng.uniform(0, 1, shape).astype(np.float32)
    ct = rng.uniform(0, 1, shape).astype(np.float32)
    eigs = rng.uniform(0.01, 2, shape + (3,)) if pointwise else (1.0, 10 ** -1.5, 10 ** -1.5)
    lab = rng.randint(0, 3, shape).astype(np.uint8) if supervised else None
    for sc in [(1, 1, 1), (1.5, 0.7, 1.2)]:
        a = O.maxflow_solve(img, q, eigs, alpha, cs, ct, labels=lab, scaling=sc, num_iter=30, update=4,
                            error_bound=-1)
        b = O.ref_maxflow_solve(img, q, eigs, alpha, cs, ct, labels=lab, scaling=sc, num_iter=30, update=4,
                                error_bound=-1)
        assert a[1] == b[1]
        assert _bits_equal(a[0], b[0])


def test_sum_abs_matches_numpy():
    rng = np.random.RandomState(3)
    for n in [1, 5, 1024, 1025, 4097, 100000]:
        x = rng.normal(size=n).astype(np.float32)
        assert abs(O.sum_abs(x) - np.abs(x.astype(np.float64)).sum()) <= 1e-5 * max(1.0, np.abs(x).sum())


def test_nan_image_stops_at_first_check():
    rng = np.random.RandomState(4)
    shape = (6, 6, 6)
    img = rng.normal(size=shape).astype(np.float32)
    img[2, 2, 2] = np.nan
    q = I.random_squeezed(rng, shape)
    one = np.ones(shape, np.float32)
    u, iters, resid = O.maxflow_solve(img, q, (1, 1, 1), 0.1, one, one, num_iter=50, update=5, error_bound=1e-4)
    assert iters == 1 and np.isnan(resid[0])
