"""The per-volume cut inputs and the fast Dice score on the GPU
(csrc/capacities.cu) against the host restatements of the reference
experiment (miccai2016_gb300/phantom.py: bgfg_weights, grad_mag_sq,
fast_dice; src/phantom_experiment.py:38-49, 280-301, 345).  float64 on both
sides, rounded to float32: at most 2 ulp apart (CUDA's and numpy's exp/log
differ in the last bits of a double); |grad I|^2 bit-exact."""
import numpy as np
import pytest

from miccai2016_gb300 import phantom as P

pytestmark = pytest.mark.gpu


def _ulps(a, b):
    a = np.ascontiguousarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.ascontiguousarray(b, np.float32).view(np.int32).astype(np.int64)
    return int(np.max(np.abs(a - b))) if a.size else 0


@pytest.mark.parametrize("shape,sigma", [((24, 31, 40), 1.5), ((2, 2, 2), 0.1), ((64, 64, 64), 0.8),
                                         ((5, 130, 3), 1.0)])
def test_capacities_match_the_host_code(shape, sigma):
    from miccai2016_gb300.capacities import cut_inputs
    noisy, _ = P.helix_phantom(shape, 2.0, min(shape) * 0.25, 12.0, sigma, seed=3)
    fgw, bgw, g2 = cut_inputs(noisy, sigma)
    hb, hf = P.bgfg_weights(noisy, sigma)
    assert _ulps(fgw, hf.astype(np.float32)) <= 2
    assert _ulps(bgw, hb.astype(np.float32)) <= 2
    assert np.array_equal(g2, P.grad_mag_sq(noisy).astype(np.float32))


def test_capacities_on_device_tensors_and_without_grad2():
    import torch
    from miccai2016_gb300.capacities import cut_inputs
    noisy, _ = P.helix_phantom((20, 22, 24), 2.0, 5.0, 10.0, 1.2, seed=1)
    f1, b1, g1 = cut_inputs(noisy, 1.2)
    f2, b2, g2 = cut_inputs(torch.from_numpy(noisy).cuda(), 1.2, want_grad2=False)
    assert g2 is None and f2.is_cuda
    assert np.array_equal(f1, f2.cpu().numpy()) and np.array_equal(b1, b2.cpu().numpy())


def test_gradient_needs_two_voxels_per_axis():
    from miccai2016_gb300 import _native as N
    from miccai2016_gb300.capacities import cut_inputs
    with pytest.raises(N.M16Error):
        cut_inputs(np.zeros((1, 8, 8), np.float32), 1.0)
    f, b, g = cut_inputs(np.zeros((1, 8, 8), np.float32), 1.0, want_grad2=False)
    assert f.shape == (1, 8, 8) and g is None


def test_fast_dice_many_segmentations():
    import torch
    from miccai2016_gb300.capacities import fast_dice
    rng = np.random.RandomState(0)
    truth = (rng.uniform(size=(30, 40, 50)) < 0.1).astype(np.float32)
    segs = [rng.normal(0.4, 0.3, truth.shape).astype(np.float32) + 0.3 * truth * k for k in range(5)]
    got = fast_dice([torch.from_numpy(s).cuda() for s in segs], truth)
    want = [P.fast_dice(s, truth) for s in segs]
    assert np.max(np.abs(np.asarray(got) - np.asarray(want))) <= 1e-9
    assert abs(fast_dice(segs[2], truth) - want[2]) <= 1e-9
    assert fast_dice(truth, truth) == 1.0
