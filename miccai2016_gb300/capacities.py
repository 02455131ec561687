"""
The per-volume cut inputs and the fast Dice score on the GPU
(csrc/capacities.cu): the replacements of the reference experiment's host
steps _calculate_bgfg_weights_for (src/phantom_experiment.py:280-301),
np.linalg.norm(np.gradient(img), axis=0) ** 2 (:345) and fast_dice_for
(:38-49).  numpy in, numpy out; CUDA torch tensors in, CUDA tensors out.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N

EPS_REG = 1e-9   # PhantomExperiment.eps_reg (phantom_experiment.py:153)


def cut_inputs(img, noise_level, eps=EPS_REG, want_grad2=True):
    """(fgw, bgw, grad2) float32: the source capacities (foreground weights),
    the sink capacities (background weights) and |grad img|^2."""
    torch = N.torch_mod()
    on_device = N.is_torch(img)
    shape = tuple(int(s) for s in img.shape)
    if len(shape) != 3:
        raise ValueError("img must be three-dimensional")
    d = N.to_device_f32(img, shape)
    fgw = torch.empty(shape, dtype=torch.float32, device=N.device())
    bgw = torch.empty_like(fgw)
    g2 = torch.empty_like(fgw) if want_grad2 else None
    st = N.lib().m16_capacities(N.ptr(d), shape[0], shape[1], shape[2], float(noise_level), float(eps), N.ptr(fgw),
                                N.ptr(bgw), N.ptr(g2), N.stream_ptr())
    N.check("m16_capacities", st)
    out = (fgw, bgw, g2)
    if on_device:
        return out
    return tuple(None if t is None else t.cpu().numpy() for t in out)


def fast_dice(segmentations, ground_truth):
    """Fast Dice of one or many segmentations (CUDA tensors or numpy arrays of
    the ground truth's shape) against the ground truth; a float or a list."""
    L = N.lib()
    single = N.is_torch(segmentations) or isinstance(segmentations, np.ndarray)
    segs = [segmentations] if single else list(segmentations)
    truth = N.to_device_f32(ground_truth)
    n = truth.numel()
    dev = [N.to_device_f32(s) for s in segs]
    for s in dev:
        if s.numel() != n:
            raise ValueError("segmentation and ground truth differ in size")
    ptrs = (ctypes.c_void_p * len(dev))(*[s.data_ptr() for s in dev])
    out = (ctypes.c_double * len(dev))()
    ws = N.workspace(L.m16_fast_dice_workspace_bytes(len(dev)))
    st = L.m16_fast_dice(ptrs, len(dev), n, N.ptr(truth), out, N.ptr(ws), ws.numel(), N.stream_ptr())
    N.check("m16_fast_dice", st)
    vals = [float(v) for v in out]
    return vals[0] if single else vals
