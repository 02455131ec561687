"""
Ridge detection in a vesselness response -- the drop-in for the reference
module of the same name (src/processing/ridge_detection.py).

RawRidgeDetector runs the in-plane local-maximum test on the GPU
(m16_detect_ridges, csrc/directions.cu); hysteresis_threshold labels the
candidates' 26-connected components once (on the GPU by default).
"""
from __future__ import annotations

import numpy as np

from . import _native as N


class RawRidgeDetector(object):
    """ridge_detection.py:12-77: ridge candidates are voxels whose response is
    above `threshold` and above its 8 neighbours in the plane of the second
    and third eigenvectors."""

    def __init__(self, loader, threshold):
        self.__threshold = threshold
        self._dtype = np.float32
        self._loader = loader  # accepted for compatibility, unused
        self._shape = None

    @property
    def threshold(self):
        return self.__threshold

    def execute(self, result_buffer, response_buffer, qeigs_buffer, shape):
        """Device-buffer form of the reference call: result_buffer (N float32),
        response_buffer (N float32) and qeigs_buffer (N x 3 squeezed
        quaternions) are CUDA torch tensors; the result is written in place."""
        assert len(shape) == 3
        n = int(np.prod(shape))
        assert result_buffer.numel() >= n and response_buffer.numel() >= n and qeigs_buffer.numel() >= 3 * n
        st = N.lib().m16_detect_ridges(N.ptr(response_buffer), N.ptr(qeigs_buffer), int(shape[0]), int(shape[1]),
                                       int(shape[2]), float(self.threshold), N.ptr(result_buffer), N.stream_ptr())
        N.check("m16_detect_ridges", st)

    def detect(self, response, qeigs):
        """numpy/torch in, same kind out: the {0, 1} float32 ridge map."""
        torch = N.torch_mod()
        on_device = N.is_torch(response)
        shape = tuple(int(s) for s in response.shape)
        r = N.to_device_f32(response, shape)
        q = N.to_device_f32(qeigs, shape + (3,))
        out = torch.empty(shape, dtype=torch.float32, device=N.device())
        self.execute(out, r, q, shape)
        return out if on_device else out.cpu().numpy()


def hysteresis_threshold(cand, sure, labeler="gpu"):
    """ridge_detection.py:80-131: the voxels of `cand` 26-connected (through
    candidates) to a voxel of `sure`, plus `sure` itself.  As in the reference,
    `sure` is overwritten with the result and returned (and `cand` is cleared
    where the result is set).

    The reference floods from every sure voxel with an explicit stack; the
    union of its floods is exactly the union of the 26-connected components of
    (cand | sure) that contain a sure voxel, which is computed here with one
    labelling pass (labeler: "gpu", m16_label26, or "host", scipy; the same
    labels)."""
    from .labeling import label26
    assert cand.shape == sure.shape
    if labeler == "gpu":
        # labels, flags and the selection on the device (m16_hysteresis)
        torch = N.torch_mod()
        L = N.lib()
        d0, d1, d2 = (int(v) for v in cand.shape)
        dc = torch.from_numpy(np.ascontiguousarray(np.asarray(cand) != 0, dtype=np.uint8)).to(N.device())
        dsu = torch.from_numpy(np.ascontiguousarray(np.asarray(sure) != 0, dtype=np.uint8)).to(N.device())
        out = torch.empty((d0, d1, d2), dtype=torch.uint8, device=N.device())
        ws = N.workspace(L.m16_hysteresis_workspace_bytes(d0, d1, d2))
        N.check("m16_hysteresis", L.m16_hysteresis(N.ptr(dc), N.ptr(dsu), d0, d1, d2, N.ptr(out), N.ptr(ws),
                                                   ws.numel(), N.stream_ptr()))
        result = out.cpu().numpy().view(bool)
    else:
        both = np.logical_or(cand, sure)
        labels, n = label26(both, where=labeler)
        keep = np.zeros(n + 1, bool)
        keep[np.unique(labels[np.asarray(sure, bool)])] = True
        keep[0] = False
        result = keep[labels]
    sure[...] = result
    cand[result] = False
    return sure
