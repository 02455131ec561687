"""The plain pipeline of the reference experiment (src/phantom_experiment.py:326-368)
end to end on the 64^3 helix workload: helix tube radius 3, helix radius 16,
pitch 20, noise sigma 1.5 (seed 0); Frangi at sigma 1, 2, 3 with alpha = beta =
0.5; ridge thresholds (0.01, 0.3) with cleaning; GVF mu 0.2 for 100
iterations; completion; capacities; an ATV cut of 300 fixed iterations at
weighting 10^-1.25 and decay 10^1.5.

It runs once through the GPU drop-ins (pipeline.prepare_cut_inputs and
CmfCutQAnisotropicGpu) and once through the oracle chain (O.frangi,
misc.normalize, oracle/adjust.advanced_adjuster, O.gvf_run,
O.complete_transformations, the host capacities, O.maxflow_solve), and the
results must agree: u within 1e-3 max-abs, the masks at 0.5 on all but 1e-4
of the voxels, Dice within 1e-3.  The intermediate stages are compared too,
so that a failure names the stage it starts in."""
import contextlib
import io

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

U_TOL = 1e-3
MASK_FRAC = 1e-4
DICE_TOL = 1e-3


def _oracle_chain(noisy, cfg, scales, thresholds):
    from miccai2016_gb300 import phantom as P
    from miccai2016_gb300.misc import normalize
    from oracle import adjust as A
    from oracle import oracle as O
    val, quat, _ = O.frangi(noisy, scales)
    resp = normalize(val, dst_min=0.0, dst_max=1.0, perc_low=None, perc_up=None, clip=True)
    with contextlib.redirect_stdout(io.StringIO()):
        vdirs, ridge, _ = A.advanced_adjuster(quat, resp, thresholds)
    scaled = np.rollaxis(np.rollaxis(vdirs, -1) * resp, 0, vdirs.ndim)
    g, _, _ = O.gvf_run(scaled, cfg["gvf_mu"], cfg["gvf_iter"], max(1, cfg["gvf_iter"] // 10), tol=0.0,
                        normalize=False)
    quats = O.complete_transformations(g)
    bgw, fgw = P.bgfg_weights(noisy, cfg["sigma"])
    alpha = P.nonterminal_weights(P.grad_mag_sq(noisy), cfg["weighting"], cfg["decay"])
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    u, iters, _ = O.maxflow_solve(noisy, quats, P.ATV_EIGS, f(alpha), f(fgw), f(bgw), num_iter=cfg["num_iter"],
                                  update=30, error_bound=-1.0)
    return dict(resp=resp, ridge=ridge, quats=quats, u=u, iterations=iters)


def _gpu_chain(noisy, cfg, scales, thresholds):
    from miccai2016_gb300 import phantom as P
    from miccai2016_gb300.continuous_cut_anisotropic_gpu import CmfCutQAnisotropicGpu
    from miccai2016_gb300.pipeline import prepare_cut_inputs
    d, _ = prepare_cut_inputs(noisy, cfg["sigma"], scales=scales, ridge_thresholds=thresholds,
                              gvf_mu=cfg["gvf_mu"], gvf_iterations=cfg["gvf_iter"])
    alpha = P.nonterminal_weights(d["grad2"].astype(np.float64), cfg["weighting"], cfg["decay"]).astype(np.float32)
    p = CmfCutQAnisotropicGpu.CutParameters()
    p.num_iter, p.update, p.error_bound = cfg["num_iter"], 30, -1.0
    cutter = CmfCutQAnisotropicGpu(p)
    u = cutter.execute(noisy, d["quats"], P.ATV_EIGS, alpha, d["fgw"], d["bgw"], verbose=False)
    return dict(resp=d["vesselness"], quats=d["quats"], u=u, iterations=cutter.last_iterations,
                ridge_points=d["ridge_points"])


def test_plain_pipeline_64cube_matches_the_oracle_chain():
    from miccai2016_gb300 import phantom as P
    cfg = P.CONFIG_PLAIN_64
    scales, thresholds = (1, 3, 3), (0.01, 0.3)
    noisy, truth = P.helix_phantom(cfg["shape"], cfg["tube_radius"], cfg["helix_radius"], cfg["pitch"], cfg["sigma"],
                                   cfg["seed"])
    noisy = noisy.astype(np.float32)
    o = _oracle_chain(noisy, cfg, scales, thresholds)
    g = _gpu_chain(noisy, cfg, scales, thresholds)
    # stage by stage (diagnostic bounds: the tolerances of the per-stage tests)
    assert np.max(np.abs(g["resp"] - o["resp"])) <= 1e-4, "vesselness"
    assert g["ridge_points"] == int(o["ridge"].sum()), "cleaned ridge size"
    # the cut
    assert g["iterations"] == o["iterations"] == cfg["num_iter"]
    du = float(np.max(np.abs(g["u"] - o["u"])))
    mask_g, mask_o = g["u"] >= 0.5, o["u"] >= 0.5
    mask_frac = float(np.mean(mask_g != mask_o))
    dice_g, dice_o = P.fast_dice(g["u"], truth), P.fast_dice(o["u"], truth)
    assert du <= U_TOL, ("u", du)
    assert mask_frac <= MASK_FRAC, ("mask", mask_frac)
    assert abs(dice_g - dice_o) <= DICE_TOL, ("dice", dice_g, dice_o)
    assert dice_o > 0.4   # the pipeline segments the tube at all (0.50 after 300 iterations)
