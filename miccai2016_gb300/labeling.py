"""
26-connected labelling of binary volumes on the GPU (csrc/label26.cu):
the labels and count of scipy.ndimage.label(mask, structure=ones((3, 3, 3))),
which the sign adjustment's hysteresis (ridge_detection.py:80-131) and ridge
cleaning (adjust_directions.py:290-339) compute.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N

STRUCTURE26 = np.ones((3, 3, 3), dtype=int)


def label26(mask, where="gpu"):
    """(labels int32 numpy array, number of components) of a 3-D mask.
    where="gpu" runs m16_label26; where="host" runs scipy.ndimage.label
    (the same result)."""
    mask = np.asarray(mask)
    if mask.ndim != 3:
        raise ValueError("mask must be three-dimensional")
    if where == "host":
        import scipy.ndimage
        lab, n = scipy.ndimage.label(mask, structure=STRUCTURE26)
        return lab.astype(np.int32, copy=False), int(n)
    if where != "gpu":
        raise ValueError("where must be 'gpu' or 'host'")
    torch = N.torch_mod()
    L = N.lib()
    d0, d1, d2 = (int(s) for s in mask.shape)
    m = torch.from_numpy(np.ascontiguousarray(mask != 0, dtype=np.uint8)).to(N.device())
    out = torch.empty((d0, d1, d2), dtype=torch.int32, device=N.device())
    ws = N.workspace(L.m16_label26_workspace_bytes(d0, d1, d2))
    n = ctypes.c_int32(0)
    st = L.m16_label26(N.ptr(m), d0, d1, d2, N.ptr(out), ctypes.byref(n), N.ptr(ws), ws.numel(), N.stream_ptr())
    N.check("m16_label26", st)
    return out.cpu().numpy(), int(n.value)
