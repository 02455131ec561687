"""
Connected-component labelling of binary volumes on the GPU (csrc/label26.cu):
the labels and count of scipy.ndimage.label(mask, structure=ones((3, 3, 3))),
which the sign adjustment's hysteresis (ridge_detection.py:80-131) and ridge
cleaning (adjust_directions.py:290-339) compute, or with the default
6-connectivity, which the experiment's Dice of the largest component
(phantom_experiment.py:52-103) uses.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N

STRUCTURE26 = np.ones((3, 3, 3), dtype=int)


def label(mask, connectivity=26, where="gpu"):
    """(labels int32 numpy array, number of components) of a 3-D mask under
    26- or 6-connectivity (scipy.ndimage.label with a 3 x 3 x 3 structure of
    ones, or its default).  where="gpu" runs m16_label; where="host" runs
    scipy.ndimage.label (the same result)."""
    mask = np.asarray(mask)
    if mask.ndim != 3:
        raise ValueError("mask must be three-dimensional")
    if connectivity not in (6, 26):
        raise ValueError("connectivity must be 6 or 26")
    if where == "host":
        import scipy.ndimage
        lab, n = scipy.ndimage.label(mask, structure=STRUCTURE26 if connectivity == 26 else None)
        return lab.astype(np.int32, copy=False), int(n)
    if where != "gpu":
        raise ValueError("where must be 'gpu' or 'host'")
    torch = N.torch_mod()
    L = N.lib()
    d0, d1, d2 = (int(s) for s in mask.shape)
    m = torch.from_numpy(np.ascontiguousarray(mask != 0, dtype=np.uint8)).to(N.device())
    out = torch.empty((d0, d1, d2), dtype=torch.int32, device=N.device())
    ws = N.workspace(L.m16_label_workspace_bytes(d0, d1, d2))
    n = ctypes.c_int32(0)
    st = L.m16_label(N.ptr(m), d0, d1, d2, int(connectivity), N.ptr(out), ctypes.byref(n), N.ptr(ws), ws.numel(),
                     N.stream_ptr())
    N.check("m16_label", st)
    return out.cpu().numpy(), int(n.value)


def label_device(mask, connectivity=26):
    """(labels int32 CUDA tensor, number of components) of a 3-D uint8 (or
    bool) CUDA tensor mask: label() without leaving the device."""
    torch = N.torch_mod()
    L = N.lib()
    if mask.dim() != 3:
        raise ValueError("mask must be three-dimensional")
    if connectivity not in (6, 26):
        raise ValueError("connectivity must be 6 or 26")
    m = mask if mask.dtype == torch.uint8 else (mask != 0).to(torch.uint8)
    m = m.contiguous()
    d0, d1, d2 = (int(s) for s in m.shape)
    out = torch.empty((d0, d1, d2), dtype=torch.int32, device=m.device)
    ws = N.workspace(L.m16_label_workspace_bytes(d0, d1, d2))
    n = ctypes.c_int32(0)
    st = L.m16_label(N.ptr(m), d0, d1, d2, int(connectivity), N.ptr(out), ctypes.byref(n), N.ptr(ws), ws.numel(),
                     N.stream_ptr())
    N.check("m16_label", st)
    return out, int(n.value)


def label26(mask, where="gpu"):
    """label(mask, 26, where): the labelling of the sign adjustment."""
    return label(mask, 26, where)


def dice_largest(segmentation, ground_truth, threshold=0.5):
    """Dice of the largest 6-connected component of segmentation >= threshold
    against a binary ground truth (phantom_experiment.py:52-103) on the GPU
    (m16_dice_largest).  Host arrays or device tensors; returns a float (0.0
    without foreground, where the reference fails)."""
    torch = N.torch_mod()
    L = N.lib()
    seg = segmentation if N.is_torch(segmentation) else torch.from_numpy(
        np.ascontiguousarray(segmentation, dtype=np.float32))
    seg = seg.to(device=N.device(), dtype=torch.float32).contiguous()
    gt = ground_truth if N.is_torch(ground_truth) else torch.from_numpy(np.ascontiguousarray(ground_truth))
    gt = (gt.to(N.device()) != 0).to(torch.uint8).contiguous()
    if seg.dim() != 3 or tuple(gt.shape) != tuple(seg.shape):
        raise ValueError("segmentation and ground truth must be 3-D of one shape")
    d0, d1, d2 = (int(s) for s in seg.shape)
    ws = N.workspace(L.m16_dice_largest_workspace_bytes(d0, d1, d2))
    dice = ctypes.c_double(0.0)
    st = L.m16_dice_largest(N.ptr(seg), N.ptr(gt), d0, d1, d2, float(threshold), ctypes.byref(dice), None, None,
                            N.ptr(ws), ws.numel(), N.stream_ptr())
    N.check("m16_dice_largest", st)
    return float(dice.value)
