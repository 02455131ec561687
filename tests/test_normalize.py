"""misc.normalize against the reference's own normalize (src/helpers/misc.py:63-114),
executed on every branch by tests/golden/make_normalize_golden.py: min-max,
percentiles (lower, upper, both), clipping on and off, the two rescalings,
a zero range, integer data.  Bit for bit."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_normalize_golden as G  # noqa: E402


def test_normalize_matches_reference_outputs_bit_for_bit():
    from miccai2016_gb300.misc import normalize
    g = np.load(os.path.join(HERE, "golden", "normalize.npz"))
    cases = G.cases()
    assert len(cases) == len(g.files) // 2
    for name, data, kw in cases:
        assert np.array_equal(g[name + "__in"], data), name
        want = g[name + "__out"]
        got = normalize(data, **kw)
        assert got.dtype == want.dtype == np.float64, name
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), name


def test_normalize_zero_range_gives_dst_min():
    from miccai2016_gb300.misc import normalize
    out = normalize(np.full((3, 3), 7, np.float32), dst_min=0.25, dst_max=2.0)
    assert out.dtype == np.float64 and np.all(out == 0.25)
