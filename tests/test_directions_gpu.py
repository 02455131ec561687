"""Parity of the CUDA direction kernels (csrc/directions.cu) and of the
drop-in AdvancedAdjuster / TransformationCompleter with the oracle.

The kernels follow the reference's rounding sequence (no contracted
multiply-adds, the quaternion expansion's cos/sin rounded to float from the
exact values), so the discrete outputs are compared exactly: main directions
and ridge maps bit for bit (a few tests allow 1e-4 of the voxels), and the
sign flips bit-exact given identical ridge inputs.  Completed frames are compared as
rotations (1e-5)."""
import io
import contextlib
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import inputs as I  # noqa: E402
from oracle import adjust as A  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _rot(sq):
    phi, th, psi = [sq[..., k].astype(np.float64) for k in range(3)]
    w = np.cos((phi + psi) / 2) * np.cos(th / 2)
    x = np.cos((phi - psi) / 2) * np.sin(th / 2)
    y = np.sin((phi - psi) / 2) * np.sin(th / 2)
    z = np.sin((phi + psi) / 2) * np.cos(th / 2)
    return np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                     2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                     2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1).reshape(-1, 3, 3)


def _gpu_adjust(vecs, coords, rdirs, scaling):
    import ctypes
    import torch
    from miccai2016_gb300 import _native as N
    d = torch.from_numpy(np.ascontiguousarray(vecs)).cuda()
    c = torch.from_numpy(np.ascontiguousarray(coords, np.uint16).view(np.int16)).cuda()
    r = torch.from_numpy(np.ascontiguousarray(rdirs)).cuda()
    sc = (ctypes.c_double * 3)(*scaling)
    st = N.lib().m16_adjust_nonridge_signs(N.ptr(d), *vecs.shape[:3], N.ptr(c), N.ptr(r), len(coords), sc,
                                          N.stream_ptr())
    N.check("m16_adjust_nonridge_signs", st)
    return d.cpu().numpy()


def _gpu_extract(q):
    import torch
    from miccai2016_gb300 import _native as N
    d = torch.from_numpy(np.ascontiguousarray(q)).cuda()
    st = N.lib().m16_extract_main_directions(N.ptr(d), d.numel() // 3, N.ptr(d), N.stream_ptr())
    N.check("m16_extract_main_directions", st)
    return d.cpu().numpy()


def test_golden_direction_kernels():
    from miccai2016_gb300.adjust_directions import TransformationCompleter
    from miccai2016_gb300.ridge_detection import RawRidgeDetector
    d = I.directions_case()
    g = np.load(os.path.join(HERE, "golden", "directions.npz"))
    for th in (0.01, 0.3):
        r = RawRidgeDetector(None, th).detect(d["resp"], d["quats"])
        assert np.mean(r != g["ridge_%g" % th]) <= 1e-4
    assert np.max(np.abs(_gpu_extract(d["quats"]) - g["main"])) <= 1e-6
    comp = TransformationCompleter(d["vecs"]).complete()
    assert np.max(np.abs(_rot(comp) - _rot(g["complete"]))) <= 1e-5
    assert np.array_equal(_bits(_gpu_adjust(d["vecs"], d["coords"], d["rdirs"], (1, 1, 1))), _bits(g["adjust_iso"]))
    assert np.array_equal(_bits(_gpu_adjust(d["vecs"], d["coords"], d["rdirs"], (1.5, 0.7, 1.2))),
                          _bits(g["adjust_aniso"]))


@pytest.mark.parametrize("shape", [(40, 33, 50), (7, 64, 3), (1, 20, 20)])
def test_kernels_match_oracle_on_random_inputs(shape):
    from miccai2016_gb300.ridge_detection import RawRidgeDetector
    rng = np.random.RandomState(sum(shape))
    resp = rng.uniform(0, 1, shape).astype(np.float32)
    q = I.random_squeezed(rng, shape)
    r = RawRidgeDetector(None, 0.05).detect(resp, q)
    assert np.mean(r != O.detect_ridges(resp, q, 0.05)) <= 1e-4
    assert np.max(np.abs(_gpu_extract(q) - O.extract_main_directions(q))) <= 1e-6
    v = rng.normal(size=shape + (3,)).astype(np.float32)
    R = 300
    coords = np.stack([rng.randint(0, s, R) for s in shape], -1).astype(np.uint16)
    rd = rng.normal(size=(R, 3)).astype(np.float32)
    for sc in [(1, 1, 1), (0.5, 2.0, 1.25)]:
        assert np.array_equal(_bits(_gpu_adjust(v, coords, rd, sc)), _bits(O.adjust_nonridge_signs(v, coords, rd, sc)))


def test_main_directions_and_ridges_bit_exact_on_a_million_quaternions():
    """The quaternion expansion's cos/sin are the floats nearest to the exact
    values (single-precision double-float evaluation, double precision where
    that is not certain): main directions and ridge maps equal the oracle's
    bit for bit over 1M voxels, including angles beyond [-4, 4] (the double
    path), half angles at and next to multiples of pi/2, and tiny angles."""
    from miccai2016_gb300.ridge_detection import RawRidgeDetector
    rng = np.random.RandomState(11)
    shape = (64, 128, 128)
    q = I.random_squeezed(rng, shape).reshape(-1, 3)
    n = len(q)
    wide = rng.rand(n) < 0.01
    q[wide] = rng.uniform(-20, 20, (int(wide.sum()), 3)).astype(np.float32)
    quarter = np.float32(np.pi / 2) * rng.randint(-2, 3, 4096).astype(np.float32)
    near = np.nextafter(quarter, np.float32(np.inf) * rng.choice([-1, 1], 4096).astype(np.float32))
    q[:4096, 1] = 2 * near
    q[4096:8192, 0] = near
    q[8192:12288, 2] = rng.uniform(-1e-5, 1e-5, 4096).astype(np.float32)
    q = q.reshape(shape + (3,))
    assert np.array_equal(_bits(_gpu_extract(q)), _bits(O.extract_main_directions(q)))
    resp = rng.uniform(0, 1, shape).astype(np.float32)
    assert np.array_equal(RawRidgeDetector(None, 0.05).detect(resp, q), O.detect_ridges(resp, q, 0.05))


def test_nearest_ridge_ties_go_to_the_lowest_index():
    shape = (1, 1, 5)
    v = np.tile(np.array([1, 0, 0], np.float32), (1, 1, 5, 1))
    coords = np.array([[0, 0, 0], [0, 0, 4], [0, 0, 2]], np.uint16)
    rd = np.array([[1, 0, 0], [-1, 0, 0], [-1, 0, 0]], np.float32)
    out = _gpu_adjust(v, coords, rd, (1, 1, 1))
    # voxel 1 is equidistant (1) from points 0 and 2 -> point 0 wins, keeps its sign
    # voxel 3 is equidistant from points 1 and 2 -> point 1 wins, flips
    assert out[0, 0, 1, 0] == 1 and out[0, 0, 3, 0] == -1
    assert np.array_equal(_bits(out), _bits(O.adjust_nonridge_signs(v, coords, rd, (1, 1, 1))))


def _small_tube():
    from miccai2016_gb300 import phantom as P
    noisy, truth = P.helix_phantom((32, 40, 40), 2.0, 10.0, 16.0, 0.3, 7)
    val, quat, _ = O.frangi(noisy, (1, 2, 2))
    resp = ((val - val.min()) / (val.max() - val.min())).astype(np.float32)
    return resp, quat


def test_advanced_adjuster_matches_oracle():
    from miccai2016_gb300.adjust_directions import AdvancedAdjuster
    resp, quat = _small_tube()
    th = (0.2, 0.5)
    with contextlib.redirect_stdout(io.StringIO()):
        adj_o, ridge_o, main_o = A.advanced_adjuster(quat, resp, th)
        obj = AdvancedAdjuster(th, quat, resp, voxel_size=(1, 1, 1))
        adj = obj.execute(verbose=False)
    assert 0 < ridge_o.sum() < 3000
    same_main = _bits(obj.main_dirs_unadjusted) == _bits(main_o)
    assert np.mean(~same_main) <= 1e-4
    assert np.max(np.abs(obj.main_dirs_unadjusted - main_o)) <= 1e-6
    assert np.mean(obj.ridge != ridge_o) <= 1e-4
    # end to end, the main directions may differ in the last bit (the
    # device's double sin/cos); the signs are compared bit for bit, on
    # identical inputs, by test_advanced_adjuster_signs_bit_exact_from_the_oracle_ridge
    assert adj.shape == adj_o.shape


class _AdjusterFromOracleRidge(object):
    """The GPU AdvancedAdjuster started from the oracle's ridge map (after the
    hysteresis) and the oracle's main directions, so that the steps after
    them -- cleaning, ridge MST, sign propagation, nearest-ridge flip -- run
    on identical inputs and every sign must come out bit for bit."""

    @staticmethod
    def make(th, quat, resp, ridge_h, main):
        import torch
        from miccai2016_gb300 import _native as N
        from miccai2016_gb300.adjust_directions import AdvancedAdjuster

        class Adj(AdvancedAdjuster):
            def _label_ridge_dev(self):
                self._d_main = torch.from_numpy(np.ascontiguousarray(main)).to(N.device())
                return torch.from_numpy(np.ascontiguousarray(ridge_h != 0, dtype=np.uint8)).to(N.device())

        return Adj(th, quat, resp, voxel_size=(1, 1, 1))


@pytest.mark.parametrize("th", [(0.2, 0.5), (0.05, 0.3)])
def test_advanced_adjuster_signs_bit_exact_from_the_oracle_ridge(th):
    resp, quat = _small_tube()
    stages = {}
    with contextlib.redirect_stdout(io.StringIO()):
        adj_o, ridge_o, main_o = A.advanced_adjuster(quat, resp, th, stages=stages)
        obj = _AdjusterFromOracleRidge.make(th, quat, resp, stages["ridge_hysteresis"], main_o)
        adj = obj.execute(verbose=False)
    assert ridge_o.sum() > 0
    assert np.array_equal(obj.ridge, ridge_o)                  # the cleaning keeps the same segments
    assert np.array_equal(_bits(adj), _bits(adj_o))            # every sign, every bit


def test_device_and_host_sequences_give_the_same_bits():
    """execute() keeps the volumes on the device by default; the host
    sequence (labelling and the MST's local phase on the host) gives the
    same ridge and the same adjusted directions, bit for bit."""
    from miccai2016_gb300.adjust_directions import AdvancedAdjuster
    resp, quat = _small_tube()
    for th, clean in (((0.05, 0.3), True), ((0.2, 0.5), False), (0.1, True)):
        with contextlib.redirect_stdout(io.StringIO()):
            dev = AdvancedAdjuster(th, quat, resp, voxel_size=(1, 1, 1), clean_ridge=clean)
            a_dev = dev.execute(verbose=False)
            host = AdvancedAdjuster(th, quat, resp, voxel_size=(1, 1, 1), clean_ridge=clean)
            host.labeler, host.mst_local = "host", "host"
            a_host = host.execute(verbose=False)
        assert np.array_equal(dev.ridge, host.ridge)
        assert np.array_equal(_bits(a_dev), _bits(a_host))
        assert np.array_equal(_bits(dev.main_dirs_unadjusted), _bits(host.main_dirs_unadjusted))


def test_ridge_detection_only_and_no_cleaning():
    from miccai2016_gb300.adjust_directions import AdvancedAdjuster
    resp, quat = _small_tube()
    obj = AdvancedAdjuster(0.3, quat, resp, ridge_detection_only=True, clean_ridge=False)
    assert obj.execute(verbose=False) is None
    assert np.mean(obj.ridge != O.detect_ridges(resp, quat, 0.3)) <= 1e-4


def test_completion_of_near_axis_directions_matches_the_oracle():
    # Near-axis directions give diagonal terms around and far below 2^-27:
    # mat2quat's 1 + m00 - m11 - m22 takes the exact integer sum above that
    # size and the double expression below it.  Rotations within 1e-5 of the
    # oracle's (the squeeze's atan2/acos differ in the last bits between libm
    # and CUDA), with the main direction kept.
    from miccai2016_gb300.adjust_directions import TransformationCompleter
    rng = np.random.RandomState(27)
    vs = []
    for t in (1e-12, 1e-9, 7.450580596923828125e-9, 7.5e-9, 3e-8, 1e-6, 2.0 ** -26, 2.0 ** -28):
        for sgn in ((1, 1, 1), (1, -1, 1), (-1, 1, -1), (-1, -1, -1)):
            for perm in ((0, 1, 2), (1, 2, 0), (2, 0, 1), (0, 2, 1), (1, 0, 2), (2, 1, 0)):
                vs.append((np.array([1.0, t, 0.37 * t])[list(perm)] * np.array(sgn)))
    v = np.concatenate([np.array(vs), rng.normal(size=(4000, 3)) * np.array([1, 1e-8, 1e-8]),
                        rng.normal(size=(4000, 3)) * np.array([1e-9, 1, 1e-7])]).astype(np.float32)
    v = v[:8000].reshape(20, 20, 20, 3)
    q = TransformationCompleter(v).complete()
    assert np.max(np.abs(_rot(q) - _rot(O.complete_transformations(v)))) <= 1e-5
    vn = v / np.linalg.norm(v.astype(np.float64), axis=-1, keepdims=True)
    assert np.max(np.abs(_gpu_extract(q) - vn)) <= 1e-5


def test_completer_round_trip_keeps_the_main_direction():
    from miccai2016_gb300.adjust_directions import TransformationCompleter
    rng = np.random.RandomState(9)
    v = rng.normal(size=(10, 11, 12, 3)).astype(np.float32)
    q = TransformationCompleter(v).complete()
    back = _gpu_extract(q)
    vn = v / np.linalg.norm(v, axis=-1, keepdims=True)
    assert np.max(np.abs(back - vn)) <= 1e-5


@pytest.mark.parametrize("shape", [(40, 33, 50), (1, 20, 20)])
def test_fused_ridges_and_main_directions_equal_the_two_calls(shape):
    import torch
    from miccai2016_gb300 import _native as N
    from miccai2016_gb300.ridge_detection import RawRidgeDetector
    rng = np.random.RandomState(sum(shape) + 1)
    resp = rng.uniform(0, 1, shape).astype(np.float32)
    q = I.random_squeezed(rng, shape)
    ridge = RawRidgeDetector(None, 0.05).detect(resp, q)
    main = _gpu_extract(q)
    d_resp = torch.from_numpy(resp).cuda()
    for in_place in (False, True):
        d_q = torch.from_numpy(np.ascontiguousarray(q)).cuda()
        d_ridge = torch.empty(shape, dtype=torch.float32, device="cuda")
        d_dirs = d_q if in_place else torch.empty_like(d_q)
        st = N.lib().m16_detect_ridges_main_directions(N.ptr(d_resp), N.ptr(d_q), *shape, 0.05, N.ptr(d_ridge),
                                                      N.ptr(d_dirs), N.stream_ptr())
        N.check("m16_detect_ridges_main_directions", st)
        assert np.array_equal(d_ridge.cpu().numpy(), ridge)
        assert np.array_equal(_bits(d_dirs.cpu().numpy()), _bits(main))
