"""The GVF oracle (oracle/gvf.c) against golden fixtures from the reference's
gvf.cl, and live against it where the reference checkout is present."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from oracle import oracle as O  # noqa: E402
import inputs as I  # noqa: E402


@pytest.mark.parametrize("name", I.GVF_CASES)
def test_oracle_matches_golden(name):
    v, kw = I.gvf_case(name)
    gold = np.load(os.path.join(HERE, "golden", name + ".npz"))
    g, iters, mags = O.gvf_run(v, **kw)
    assert iters == int(gold["iterations"])
    assert np.array_equal(g.view(np.uint32), gold["g"].view(np.uint32))
    np.testing.assert_allclose(mags, gold["mags"], rtol=1e-6)


def test_tol_case_stops_early():
    v, kw = I.gvf_case("gvf_tol")
    gold = np.load(os.path.join(HERE, "golden", "gvf_tol.npz"))
    assert int(gold["iterations"]) < kw["maxiter"]


def test_time_step_matches_formula():
    for vs, mu in [((1, 1, 1), 0.2), ((1, 1, 1), 10 ** 0.5), ((0.5, 2, 1), 1.0)]:
        ref = min(0.99, min(vs) ** 3 / (2.01 ** 3 * mu))
        assert O.gvf_time_step(vs, mu) == pytest.approx(ref, rel=1e-15)


@pytest.mark.parametrize("shape", [(2, 3, 4), (5, 7, 9), (4, 1, 6)])
def test_oracle_matches_reference_kernels(has_ref, shape):
    if not has_ref:
        pytest.skip("reference checkout not present")
    if 1 in shape:
        pytest.skip("the reference reads outside the buffer on a length-1 axis")
    rng = np.random.RandomState(sum(shape))
    v = (rng.normal(size=shape + (3,)) * 0.5).astype(np.float32)
    for mu, vs, norm in [(0.2, None, False), (10 ** 0.5, (1.5, 0.8, 1.1), True)]:
        a = O.gvf_run(v, mu, 25, 4, normalize=norm, voxel_size=vs)
        b = O.ref_gvf_run(v, mu, 25, 4, normalize=norm, voxel_size=vs)
        assert a[1] == b[1]
        assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
