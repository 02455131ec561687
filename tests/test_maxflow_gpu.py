"""Parity of the CUDA max-flow (csrc/maxflow.cu via the drop-in
CmfCutQAnisotropicGpu and the C ABI) with the oracle and the golden fixtures.

Tolerances (floating point; the CUDA path computes in fp32 with the
expanded quaternion's rotation matrix instead of the reference's double
products and two Hamilton products):
  u within 1e-3 max-abs after a fixed iteration count,
  masks u >= 0.5 differing on at most 1e-4 of the voxels,
  fast Dice within 1e-3.
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

U_TOL = 1e-3
MASK_FRAC = 1e-4
DICE_TOL = 1e-3


def _cutter(num_iter, update, error_bound, cc=0.2, steps=0.11):
    from miccai2016_gb300.continuous_cut_anisotropic_gpu import CmfCutQAnisotropicGpu
    p = CmfCutQAnisotropicGpu.CutParameters()
    p.num_iter, p.update, p.error_bound, p.cc, p.steps = num_iter, update, error_bound, cc, steps
    return CmfCutQAnisotropicGpu(p)


PATHS = ["default", "two_sweeps"]


def _path_code(path):
    from miccai2016_gb300 import _native as N
    return {"default": N.PATH_DEFAULT, "two_sweeps": N.PATH_TWO_SWEEPS}[path]


def _run_gpu(inp, kw, path="default"):
    c = _cutter(kw["num_iter"], kw["update"], kw["error_bound"])
    c.iteration_path = _path_code(path)
    u = c.execute(inp["img"], inp["quats"], inp["eigs"], inp["alpha"], inp["cs"], inp["ct"],
                  labels=inp["labels"], scaling=inp["scaling"], verbose=False)
    return u, c.last_iterations, c.last_residuals


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("name", I.MAXFLOW_CASES)
def test_golden_fixtures(name, path):
    inp, kw = I.maxflow_case(name)
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    u, iters, resid = _run_gpu(inp, kw, path)
    assert u.dtype == np.float32 and u.shape == g["u"].shape
    if kw["error_bound"] < 0:
        assert iters == int(g["iterations"])
    else:
        assert abs(iters - int(g["iterations"])) <= kw["update"]
    n = min(len(resid), len(g["residuals"]))
    np.testing.assert_allclose(resid[:n], g["residuals"][:n], rtol=1e-3, atol=1e-7)
    if iters == int(g["iterations"]):
        assert np.max(np.abs(u - g["u"])) <= U_TOL


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 6, 1), (5, 7, 9), (3, 1, 70), (33, 9, 40), (70, 3, 5)])
@pytest.mark.parametrize("supervised", [False, True])
@pytest.mark.parametrize("pointwise", [False, True])
@pytest.mark.parametrize("path", PATHS)
def test_random_variants_match_oracle(shape, supervised, pointwise, path):
    rng = np.random.RandomState(abs(hash((shape, supervised, pointwise))) % 2 ** 31)
    img = rng.normal(0.5, 0.5, shape).astype(np.float32)
    q = I.random_squeezed(rng, shape)
    alpha = rng.uniform(0.01, 0.5, shape).astype(np.float32)
    cs = rng.uniform(0, 1, shape).astype(np.float32)
    ct = rng.uniform(0, 1, shape).astype(np.float32)
    eigs = rng.uniform(0.01, 2, shape + (3,)) if pointwise else (1.0, 10 ** -1.5, 10 ** -1.5)
    lab = rng.randint(0, 3, shape).astype(np.uint8) if supervised else None
    sc = (1.5, 0.7, 1.2) if (shape[0] % 2) else (1, 1, 1)
    inp = dict(img=img, quats=q, eigs=eigs, alpha=alpha, cs=cs, ct=ct, labels=lab, scaling=sc)
    kw = dict(num_iter=100, update=10, error_bound=-1.0)
    u, iters, _ = _run_gpu(inp, kw, path)
    ru, riters, _ = O.maxflow_solve(img, q, eigs, alpha, cs, ct, labels=lab, scaling=sc, **kw)
    assert iters == riters == 100
    assert np.max(np.abs(u - ru)) <= U_TOL


def _helix_inputs(cfg):
    from miccai2016_gb300 import phantom as P
    return P.maxflow_inputs(cfg)


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("eigs_name", ["atv", "tv"])
def test_helix_64_fixed_iterations_parity(eigs_name, path):
    """The plain 64^3 configuration: 300 fixed iterations, ATV and TV."""
    from miccai2016_gb300 import phantom as P
    cfg = P.CONFIG_PLAIN_64
    eigs = P.ATV_EIGS if eigs_name == "atv" else P.TV_EIGS
    noisy, truth, quats, ntw, fgw, bgw = _helix_inputs(cfg)
    c = _cutter(cfg["num_iter"], 30, -1.0)
    c.iteration_path = _path_code(path)
    u = c.execute(noisy, quats, eigs, ntw, fgw, bgw, labels=None, scaling=(1, 1, 1), verbose=False)
    ru, riters, _ = O.maxflow_solve(noisy, quats, eigs, ntw, fgw, bgw, num_iter=cfg["num_iter"], update=30,
                                    error_bound=-1.0)
    assert c.last_iterations == riters == cfg["num_iter"]
    assert np.max(np.abs(u - ru)) <= U_TOL
    assert np.mean((u >= 0.5) != (ru >= 0.5)) <= MASK_FRAC
    assert abs(P.fast_dice(u, truth) - P.fast_dice(ru, truth)) <= DICE_TOL
    if eigs_name == "atv":
        assert P.fast_dice(u, truth) > 0.3


def test_helix_256_against_the_oracle():
    """The 256^3 configuration (tube 12, helix 64, pitch 80, noise 1.0) for
    20 fixed iterations against the oracle, plus the first residual checks
    (update 10) -- the size the headline solve runs at."""
    from miccai2016_gb300 import phantom as P
    cfg = P.CONFIG_PLAIN_256
    noisy, truth, quats, ntw, fgw, bgw = _helix_inputs(cfg)
    kw = dict(num_iter=20, update=10, error_bound=-1.0)
    c = _cutter(**kw)
    u = c.execute(noisy, quats, P.ATV_EIGS, ntw, fgw, bgw, verbose=False)
    ru, riters, rres = O.maxflow_solve(noisy, quats, P.ATV_EIGS, ntw, fgw, bgw, **kw)
    assert c.last_iterations == riters == 20
    assert np.max(np.abs(u - ru)) <= U_TOL
    assert np.mean((u >= 0.5) != (ru >= 0.5)) <= MASK_FRAC
    np.testing.assert_allclose(c.last_residuals, rres, rtol=1e-4)


@pytest.mark.parametrize("path", PATHS)
def test_residual_stop_matches_oracle(path):
    from miccai2016_gb300 import phantom as P
    cfg = P.CONFIG_PLAIN_64
    noisy, truth, quats, ntw, fgw, bgw = _helix_inputs(cfg)
    kw = dict(num_iter=3000, update=30, error_bound=1e-3)
    c = _cutter(**kw)
    c.iteration_path = _path_code(path)
    u = c.execute(noisy, quats, P.ATV_EIGS, ntw, fgw, bgw, verbose=False)
    ru, riters, rres = O.maxflow_solve(noisy, quats, P.ATV_EIGS, ntw, fgw, bgw, **kw)
    assert riters < kw["num_iter"]
    assert abs(c.last_iterations - riters) <= kw["update"]
    n = min(len(rres), len(c.last_residuals))
    np.testing.assert_allclose(c.last_residuals[:n], rres[:n], rtol=1e-2)
    if c.last_iterations == riters:
        assert np.max(np.abs(u - ru)) <= U_TOL


def test_device_tensors_give_the_same_bits_as_numpy():
    import torch
    inp, kw = I.maxflow_case("mf_const_unsup")
    u_np, _, _ = _run_gpu(inp, kw)
    c = _cutter(kw["num_iter"], kw["update"], kw["error_bound"])
    dev = {k: torch.from_numpy(np.ascontiguousarray(inp[k])).cuda() for k in ("img", "quats", "alpha", "cs", "ct")}
    u_t = c.execute(dev["img"], dev["quats"], inp["eigs"], dev["alpha"], dev["cs"], dev["ct"], verbose=False)
    assert isinstance(u_t, torch.Tensor) and u_t.is_cuda
    assert np.array_equal(u_t.cpu().numpy().view(np.uint32), u_np.view(np.uint32))


def test_nan_input_stops_at_first_check():
    rng = np.random.RandomState(5)
    shape = (8, 8, 8)
    img = rng.normal(size=shape).astype(np.float32)
    img[3, 3, 3] = np.nan
    q = I.random_squeezed(rng, shape)
    one = np.ones(shape, np.float32)
    c = _cutter(50, 5, 1e-4)
    c.execute(img, q, (1, 1, 1), 0.1, one, one, verbose=False)
    assert c.last_iterations == 1 and np.isnan(c.last_residuals[0])


def test_scalar_and_array_alpha_agree():
    inp, kw = I.maxflow_case("mf_const_unsup")
    a = dict(inp)
    a["alpha"] = 0.2
    b = dict(inp)
    b["alpha"] = np.full(inp["img"].shape, 0.2, np.float32)
    ua, _, _ = _run_gpu(a, kw)
    ub, _, _ = _run_gpu(b, kw)
    assert np.array_equal(ua, ub)


def test_removed_iteration_paths_are_rejected():
    """Only the two sweeps remain (the fused iteration and two iterations per
    launch measured slower at every size); their path values are rejected."""
    import ctypes
    from miccai2016_gb300 import _native as N
    inp, kw = I.maxflow_case("mf_const_unsup")
    c = _cutter(kw["num_iter"], kw["update"], kw["error_bound"])
    for path in (2, 3):
        c.iteration_path = path
        with pytest.raises(N.M16Error):
            c.execute(inp["img"], inp["quats"], inp["eigs"], inp["alpha"], inp["cs"], inp["ct"],
                      labels=inp["labels"], scaling=inp["scaling"], verbose=False)
