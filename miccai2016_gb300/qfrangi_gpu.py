"""
Frangi vesselness on the GPU -- the drop-in for the reference module of the
same name (src/processing/qfrangi_gpu.py).

`FeatureFilter(vesselness_params).execute_for(img, roi, voxel_size=None)`
returns `(vesselness, vesselness_dirs, slc)` exactly as the reference does:
the maximum Frangi response over the scales and, per voxel, the squeezed
quaternion of the eigenvector matrix ("eigenvectors in columns", eigenvalues
ascending by absolute value) of the scale that produced it.  All scales run in
one m16_frangi call (csrc/frangi.cu); the Gaussian derivative taps are built
here with numpy exactly as GaussianFilter3D._gauss_kernel_with does.
"""
from __future__ import annotations

import ctypes
from collections import namedtuple

import numpy as np

from . import _native as N
from .parameters import Parameters, TreePrintable

MAX_TAPS = 127


def gauss_kernel_with(sigma, order, scaling_factor=1, n_sigmas=4, round_up=False):
    """Odd-sized Gaussian derivative kernel of the given order (0-3), the
    reference's GaussianFilter3D._gauss_kernel_with (qfrangi_gpu.py:158-185)."""
    sigma_sq = sigma ** 2

    def gaussian(x):
        result = np.exp(-.5 * x ** 2 / sigma_sq)
        return result / np.sum(result)

    order0 = lambda x: gaussian(x)
    order1 = lambda x: gaussian(x) * (-x) / (sigma_sq)
    order2 = lambda x: gaussian(x) * (x ** 2 - sigma_sq) / (sigma_sq ** 2)
    order3 = lambda x: gaussian(x) * x * (3 * sigma_sq - x ** 2) / (sigma_sq ** 3)
    orders = [order0, order1, order2, order3]
    x_max = (int(np.ceil(n_sigmas * sigma)) if round_up else int(n_sigmas * sigma + 0.5))
    x_s = np.arange(-x_max, x_max + 1)
    return np.require(scaling_factor * orders[order](x_s), np.float32, ["C", "A"])


def scales_in_voxels(scales, voxel_size):
    """M x 3 per-axis sigmas [voxel] (qfrangi_gpu.py:590-592)."""
    scales_mm = np.linspace(*scales).reshape(-1, 1)
    scaling = np.divide(1., voxel_size).reshape(1, -1)
    return np.dot(scales_mm, scaling)


def pack_taps(sigmas, n_sigmas=4, round_up=False, scale_space_gamma=1):
    """(taps, radius) in the layout of m16_frangi for an M x 3 sigma array:
    orders 0, 1, 2 per axis, each scaled by sigma ** (order * gamma)."""
    sigmas = np.atleast_2d(np.asarray(sigmas, dtype=np.float64))
    m = sigmas.shape[0]
    taps = np.zeros((m, 3, 3, MAX_TAPS), np.float32)
    radius = np.zeros((m, 3), np.int32)
    for s in range(m):
        for a in range(3):
            sg = float(sigmas[s, a])
            for o in range(3):
                k = gauss_kernel_with(sg, o, sg ** (o * scale_space_gamma), n_sigmas, round_up)
                if len(k) > MAX_TAPS:
                    raise ValueError("sigma %g needs %d taps; at most %d are supported" % (sg, len(k), MAX_TAPS))
                taps[s, a, o, :len(k)] = k
                radius[s, a] = len(k) // 2
    return taps, radius


class VesselnessCalculation(object):
    """Holder of the reference's parameter class (qfrangi_gpu.py:442-468)."""

    class Parameters(Parameters):
        def __init__(self):
            self.alpha = 0.5   # weight of the lambda2 / lambda3 ratio (Frangi eqs. 11, 13)
            self.beta = 0.5    # weight of the lambda1 / sqrt(lambda2 lambda3) ratio (eqs. 10, 13)
            self.c = None      # structureness weight (eqs. 12, 13); None: half the maximum Hessian norm
            self.bright_objects = None   # True: bright tubes on a dark background
            self.scales = None  # (start [mm], stop [mm], number) of the scales


def bounding_box(mask, margin=0):
    """Slices of the bounding box of mask's non-zeros widened by margin
    (src/processing/slicing.py:13-41)."""
    margin = (np.ones(mask.ndim) * np.round(margin)).astype(int)
    i = np.nonzero(mask)
    try:
        lowers = np.maximum(0, np.min(i, axis=1) - margin)
        uppers = np.maximum(0, np.max(i, axis=1) + margin + 1)
    except ValueError:
        lowers = uppers = np.zeros(mask.ndim, dtype=int)
    return tuple(slice(int(lo), int(up), 1) for lo, up in zip(lowers, uppers))


def add_margin_to_slc(margin, slc):
    """src/processing/slicing.py:44-61"""
    d = len(slc)
    margin = (np.ones(d) * np.round(margin)).astype(int)
    arr = np.asarray([[s.start, s.stop, s.step] for s in slc])
    arr[:, 0] = arr[:, 0] - margin
    arr[:, 1] = arr[:, 1] + margin
    arr[:, :2] = np.clip(arr[:, :2], 0, np.inf)
    return tuple(slice(*[int(v) for v in row]) for row in arr)


class FeatureFilter(TreePrintable):
    """Frangi vesselness of 3D images in their regions of interest at the
    given scales (qfrangi_gpu.py:634-783)."""

    DummyBuffer = namedtuple("DummyBuffer", ["size"])

    def __init__(self, vesselness_params, loader=None, verbose=True):
        self._dtype = np.float32
        self._loader = loader  # accepted for compatibility, unused
        self.vesselness_params = vesselness_params
        self.n_sigmas = 4
        self.round_up = False   # int(4 sigma + 0.5), as scipy's gaussian_filter
        self.last_c = None
        self._ws = None

    def execute_for(self, img, roi, voxel_size=None):
        """Returns (vesselness, vesselness_dirs, slc); see the module docstring.
        CUDA torch tensors in give CUDA tensors out."""
        torch = N.torch_mod()
        L = N.lib()
        on_device = N.is_torch(img)
        voxel_size = np.ones_like(np.asarray(img.shape)) if voxel_size is None else voxel_size
        cropped, slc = self._determine_slicing_and_crop_voxels(img, roi, voxel_size)
        shape = tuple(int(s) for s in cropped.shape)
        if len(shape) != 3:
            raise ValueError("img must be three-dimensional")
        p = self.vesselness_params
        sig = scales_in_voxels(p.scales, np.multiply(voxel_size, np.ones(3)))
        taps, radius = pack_taps(sig, self.n_sigmas, self.round_up)
        d_img = N.to_device_f32(cropped, shape)
        val = torch.empty(shape, dtype=torch.float32, device=N.device())
        quat = torch.empty(shape + (3,), dtype=torch.float32, device=N.device())
        m = sig.shape[0]
        nbytes = L.m16_frangi_workspace_bytes(shape[0], shape[1], shape[2], m)
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = N.workspace(nbytes)
        c_used = (ctypes.c_float * m)()
        c = -1.0 if p.c is None else float(p.c)
        st = L.m16_frangi(N.ptr(d_img), shape[0], shape[1], shape[2], m, taps.ctypes.data_as(ctypes.c_void_p),
                          radius.ctypes.data_as(ctypes.c_void_p), float(p.alpha), float(p.beta), c,
                          int(bool(p.bright_objects)), N.ptr(val), N.ptr(quat), c_used, N.ptr(self._ws),
                          self._ws.numel(), N.stream_ptr())
        N.check("m16_frangi", st)
        self.last_c = np.array(c_used[:], np.float32)
        if on_device:
            return val, quat, slc
        return val.cpu().numpy(), quat.cpu().numpy(), slc

    def _determine_slicing_and_crop_voxels(self, voxels, roi, voxel_size):
        """qfrangi_gpu.py:755-783: crop to the ROI plus the largest kernel arm."""
        if roi is None:
            return voxels, None
        max_scales = self.vesselness_params.scales[1] / np.asarray(voxel_size, dtype=float)
        margin = (np.ceil(self.n_sigmas * max_scales) if self.round_up else
                  (self.n_sigmas * max_scales + 0.5).astype(int))
        if isinstance(roi, np.ndarray):
            roi = bounding_box(roi, margin=0)
        slc = add_margin_to_slc(margin, roi)
        return voxels[slc], slc


def hessian(img, sigma3):
    """N x 6 Hessian of one scale on the GPU (Hessian.execute, qfrangi_gpu.py:208-271)."""
    torch = N.torch_mod()
    L = N.lib()
    on_device = N.is_torch(img)
    shape = tuple(int(s) for s in img.shape)
    taps, radius = pack_taps(np.asarray(sigma3, np.float64).reshape(1, 3))
    d_img = N.to_device_f32(img, shape)
    h = torch.empty(shape + (6,), dtype=torch.float32, device=N.device())
    ws = N.workspace(L.m16_frangi_workspace_bytes(shape[0], shape[1], shape[2], 1))
    st = L.m16_hessian(N.ptr(d_img), shape[0], shape[1], shape[2], taps.ctypes.data_as(ctypes.c_void_p),
                       radius.ctypes.data_as(ctypes.c_void_p), N.ptr(h), N.ptr(ws), ws.numel(), N.stream_ptr())
    N.check("m16_hessian", st)
    return h if on_device else h.cpu().numpy()


def eigendecomposition(h6):
    """[l1, l2, l3 ascending by |l|, squeezed quaternion] of each N x 6 Hessian
    (Eigendecomposition.execute, qfrangi_gpu.py:274-332)."""
    torch = N.torch_mod()
    L = N.lib()
    on_device = N.is_torch(h6)
    d = N.to_device_f32(h6)
    out = torch.empty_like(d)
    st = L.m16_eigs(N.ptr(d), d.numel() // 6, N.ptr(out), N.stream_ptr())
    N.check("m16_eigs", st)
    return out if on_device else out.cpu().numpy()
