"""
The reference experiment's per-volume preparation of the cut inputs
(src/phantom_experiment.py:326-345), on the GPU drop-ins:

  vesselness, quaternions   FeatureFilter.execute_for      (qfrangi_gpu)
  vesselness in [0, 1]      misc.normalize
  sign-adjusted directions  AdvancedAdjuster.execute        (adjust_directions)
  smoothed directions       GvfGpu.execute on dirs * vesselness (gradient_vector_flow)
  quaternions of the cut    TransformationCompleter.complete
  capacities, |grad I|^2    Gaussian log-likelihood ratio, np.gradient (capacities.cut_inputs)

The result feeds CmfCutQAnisotropicGpu or the batched engine.
"""
from __future__ import annotations

import io
import contextlib
import time

import numpy as np

from .adjust_directions import AdvancedAdjuster, TransformationCompleter
from .capacities import cut_inputs
from .gradient_vector_flow import GvfGpu, GvfParameters
from .misc import normalize
from .qfrangi_gpu import FeatureFilter, VesselnessCalculation


def prepare_cut_inputs(img, noise_level, scales=(1, 3, 3), ridge_thresholds=(0.01, 0.3), gvf_mu=0.2,
                       gvf_iterations=100, voxel_size=(1, 1, 1), quiet=True):
    """Returns (dict of float32 host arrays: quats, fgw (= C_s), bgw (= C_t),
    grad2, vesselness; dict of stage timings in seconds)."""
    t = {}
    t0 = time.perf_counter()
    vp = VesselnessCalculation.Parameters()
    vp.bright_objects = True
    vp.scales = scales
    vesselness, vdirs_raw, _ = FeatureFilter(vp).execute_for(img, roi=None, voxel_size=voxel_size)
    vesselness = normalize(vesselness, dst_min=0.0, dst_max=1.0, perc_low=None, perc_up=None, clip=True)
    t["frangi"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    sink = io.StringIO()
    with contextlib.redirect_stdout(sink) if quiet else contextlib.nullcontext():
        adj = AdvancedAdjuster(threshold=ridge_thresholds, qeigs=vdirs_raw, response=vesselness,
                               voxel_size=voxel_size, ridge_detection_only=False, clean_ridge=True)
        vdirs = adj.execute(verbose=not quiet)
    t["adjust"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    vdirs_scaled = np.rollaxis(np.rollaxis(vdirs, -1) * vesselness, 0, vdirs.ndim)
    gp = GvfParameters()
    gp.mu, gp.tol, gp.maxiter, gp.callback = gvf_mu, 0, gvf_iterations, None
    gp.update, gp.normalize = max(1, gvf_iterations // 10), False
    vdirs_smoothed = GvfGpu(vdirs_scaled, gp, voxel_size).execute()
    t["gvf"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    quats = TransformationCompleter(vdirs_smoothed).complete()
    t["complete"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    fgw, bgw, grad2 = cut_inputs(img, noise_level)
    t["capacities"] = time.perf_counter() - t0
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    return dict(quats=f(quats), fgw=fgw, bgw=bgw, grad2=grad2, vesselness=f(vesselness),
                ridge_points=int(adj.ridge.sum())), t
