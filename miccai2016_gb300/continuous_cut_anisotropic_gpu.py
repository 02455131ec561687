"""
Continuous max-flow with anisotropic total variation (ATV) on the GPU -- the
drop-in for the reference module of the same name
(src/processing/continuous_cut_anisotropic_gpu.py).

`CmfCutQAnisotropicGpu(params).execute(img, quats, eigs, alpha, cs, ct,
labels=None, scaling=None, verbose=True)` keeps the reference's signature,
argument meaning and return value (u as a new float32 array, not clipped).
The whole solve runs in one call of m16_maxflow_solve (csrc/maxflow.cu);
ATV and TV, and every (weighting, decay), share one compiled kernel because
the reference's -D macros are runtime arguments here.

Inputs may also be CUDA torch tensors; then u is returned as a CUDA tensor
and nothing crosses PCIe.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N
from .parameters import Parameters, TreePrintable


class CmfCutQAnisotropicGpu(TreePrintable):
    """Augmented-Lagrangian continuous max-flow (paper Alg. 1.1) with the
    metric A = R diag(eigs) R^T (continuous_cut_anisotropic_gpu.py:36-344)."""

    class CutParameters(Parameters):
        """continuous_cut_anisotropic_gpu.py:38-49"""

        def __init__(self):
            self.cc = 0.2  # step size for the augmented Lagrangian
            self.error_bound = 1e-4
            self.num_iter = 1000
            self.update = 1
            self.steps = 0.11  # step size for the gradient ascent
            # Launch shapes of the reference's OpenCL kernels; kept for
            # compatibility, the CUDA kernels choose their own tiling.
            self.lsize_3d = (64, 2, 1)
            self.lsize_1d = None

    def __init__(self, params, cl_program_loader=None):
        self.float_type = np.float32
        self.float_bytes = 4
        self.params = params
        self.loader = cl_program_loader  # accepted for compatibility, unused
        self.scaling = None
        self.const_sqevals = None
        self.supervised = None
        self.rcc = None
        self.last_iterations = None
        self.last_residuals = None
        self._ws = None
        # how an iteration is launched (N.PATH_DEFAULT = N.PATH_TWO_SWEEPS)
        self.iteration_path = N.PATH_DEFAULT
        self.last_stats = None

    # -- reference: execute() with its exception-forwarding wrapper (:143-196)
    def execute(self, img, quats, eigs, alpha, cs, ct, labels=None, scaling=None, verbose=True):
        """
        <img>     3D image, used for the initialisation u = img / max(img) and for the shape
        <quats>   (z, y, x, 3) squeezed quaternions of the anisotropy's eigenvectors
        <eigs>    3 constant eigenvalues, or a (z, y, x, 3) array of per-voxel eigenvalues
        <alpha>   TV weight, scalar or (z, y, x)
        <cs>      source (foreground) capacities, (z, y, x)
        <ct>      sink (background) capacities, (z, y, x)
        <labels>  optional uint8 seeds (1 foreground, 2 background) -> supervised cut
        <scaling> voxel size [mm/voxel]; None means (1, 1, 1)
        Returns u, the relaxed labelling, as float32 of img's shape.
        """
        return self._execute(img, quats, eigs, alpha, cs, ct, labels, scaling, verbose)

    def _execute(self, img, quats, eigs, alpha, cs, ct, labels, scaling, verbose):
        torch = N.torch_mod()
        L = N.lib()
        on_device = N.is_torch(img)
        shape = tuple(int(s) for s in (img.shape if on_device else np.shape(img)))
        if len(shape) != 3:
            raise ValueError("img must be three-dimensional, got shape %s" % (shape,))
        n = int(np.prod(shape))
        scaling = (1, 1, 1) if scaling is None else tuple(float(s) for s in np.multiply(scaling, np.ones(3)))

        # eigenvalues: constant 3-tuple or per-voxel field (:216-221, 246-251)
        sqc = None
        sqp = None
        if N.is_torch(eigs):
            sqp = N.to_device_f32(torch.sqrt(eigs.to(torch.float64)), shape + (3,))
        else:
            sq = np.sqrt(np.asanyarray(eigs, dtype=np.float64))
            if sq.ndim == 1:
                if sq.shape != (3,):
                    raise ValueError("constant eigs must have 3 values")
                sqc = (ctypes.c_double * 3)(*sq.tolist())
            else:
                sqp = N.to_device_f32(sq, shape + (3,))
        self.scaling = scaling
        self.const_sqevals = np.array(list(sqc)) if sqc is not None else False
        self.supervised = labels is not None
        smin = min(scaling)
        self.rcc = 1.0 / (self.params.cc * smin ** 2)

        d_img = N.to_device_f32(img, shape)
        q = quats if N.is_torch(quats) else np.asarray(quats)
        if tuple(q.shape) != shape + (3,):
            raise ValueError("quats must have shape %s, got %s" % (shape + (3,), tuple(q.shape)))
        d_q = N.to_device_f32(q, shape + (3,))
        alpha_scalar = 0.0
        d_alpha = None
        if N.is_torch(alpha) or isinstance(alpha, np.ndarray):
            d_alpha = N.to_device_f32(alpha, shape)
        else:
            alpha_scalar = float(alpha)
        d_cs = N.to_device_f32(cs, shape)
        d_ct = N.to_device_f32(ct, shape)
        d_lab = None if labels is None else N.to_device_u8(labels).reshape(shape)
        u = torch.empty(shape, dtype=torch.float32, device=N.device())

        p = self.params
        cp = N.CutParams(float(p.cc), float(p.steps), float(p.error_bound), int(p.num_iter), int(p.update),
                         (ctypes.c_double * 3)(*scaling))
        nbytes = L.m16_maxflow_workspace_bytes(shape[0], shape[1], shape[2], ctypes.byref(cp))
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = N.workspace(nbytes)
        cap = int(p.num_iter) // max(int(p.update), 1) + 2
        resid = (ctypes.c_double * cap)()
        iters = ctypes.c_int32(0)
        nres = ctypes.c_int32(0)
        stats = N.SolveStats(0, 0, 0, 0, 0.0, 0.0, int(self.iteration_path), 0)
        st = L.m16_maxflow_solve_ex(N.ptr(d_img), N.ptr(d_q), sqc, N.ptr(sqp), N.ptr(d_alpha), alpha_scalar,
                                    N.ptr(d_cs), N.ptr(d_ct), N.ptr(d_lab), shape[0], shape[1], shape[2],
                                    ctypes.byref(cp), N.ptr(u), ctypes.byref(iters), resid, cap,
                                    ctypes.byref(nres), N.ptr(self._ws), self._ws.numel(), N.stream_ptr(),
                                    ctypes.byref(stats))
        N.check("m16_maxflow_solve_ex", st)
        self.last_stats = stats
        self.last_iterations = int(iters.value)
        self.last_residuals = np.array(resid[:min(nres.value, cap)], dtype=np.float64)
        if verbose:
            upd = max(int(p.update), 1)
            for k, err in enumerate(self.last_residuals):
                print(k * upd + 1, err)
            if self.last_residuals.size and np.isnan(self.last_residuals[-1]):
                print("Convergence criterion is NaN. Stop iterating.")
            elif self.last_residuals.size and self.last_residuals[-1] < p.error_bound:
                print("Converged.")
        if on_device:
            return u
        return u.cpu().numpy()
