"""
Gradient vector flow (Xu & Prince) on the GPU -- the drop-in for the
reference module of the same name (src/processing/gradient_vector_flow.py).

`GvfGpu(vfield, params, voxel_size=None, response=None).execute()` keeps the
reference's signature and return value ((z, y, x, 3) float32); the callback of
GvfParameters is called every `update` iterations with (field, iteration,
mean |delta|) exactly as the reference does.  The iterations run in
csrc/gvf.cu (m16_gvf_run).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N
from .parameters import Parameters


class GvfParameters(Parameters):
    """gradient_vector_flow.py:26-55: mu (regularisation), tol (stop when the
    mean |delta| falls below it), maxiter, callback(field, i, mag_delta),
    update (iterations between checks and callbacks), normalize (unit-length
    output vectors)."""

    def __init__(self):
        self.mu = None
        self.tol = None
        self.maxiter = None
        self.callback = None
        self.update = None
        self.normalize = None


def time_step_for(voxel_size, mu, ndim):
    """gradient_vector_flow.py:58-65"""
    return np.minimum(0.99, (np.min(voxel_size) ** ndim) / (2.01 ** ndim * mu))


class GvfGpu(object):
    """GVF of a 3D vector field (gradient_vector_flow.py:68-253).
    CAUTION: works for 3D only."""

    def __init__(self, vfield, params, voxel_size=None, response=None, cl_program_loader=None):
        self.ftype = np.float32
        shape = tuple(vfield.shape)
        assert len(shape) == 4 and shape[-1] == 3
        self.shape = shape[:3]
        self.n_voxels = int(np.prod(self.shape))
        self.params = params
        self.voxel_size = np.ones(3) if voxel_size is None else np.multiply(voxel_size, np.ones(3))
        self.dt = time_step_for(self.voxel_size, params.mu, ndim=3)
        self.loader = cl_program_loader  # accepted for compatibility, unused
        self._on_device = N.is_torch(vfield)
        self._v = N.to_device_f32(vfield, shape)
        self._r = None
        if response is not None:
            assert tuple(response.shape) == self.shape
            self._r = N.to_device_f32(response, self.shape)
        self.last_iterations = None
        self.last_mags = None

    def execute(self):
        torch = N.torch_mod()
        L = N.lib()
        p = self.params
        d0, d1, d2 = self.shape
        maxiter = int(p.maxiter)
        update = max(int(p.update), 1)
        tol = float(p.tol) if p.tol is not None else 0.0
        cap = maxiter // update + 2
        nbytes = L.m16_gvf_workspace_bytes(d0, d1, d2, int(self._r is not None), cap)
        ws = N.workspace(nbytes)
        g = torch.empty(self.shape + (3,), dtype=torch.float32, device=N.device())
        vs = (ctypes.c_double * 3)(*[float(v) for v in self.voxel_size])
        mags = (ctypes.c_double * cap)()
        it, stopped, nm = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int32(0)

        def run(first, count, normalize):
            st = L.m16_gvf_run(N.ptr(self._v), N.ptr(self._r), d0, d1, d2, vs, float(p.mu), float(self.dt), first,
                               count, update, tol, int(normalize), N.ptr(g), ctypes.byref(it),
                               ctypes.byref(stopped), mags, cap, ctypes.byref(nm), N.ptr(ws), ws.numel(),
                               N.stream_ptr())
            N.check("m16_gvf_run", st)

        if p.callback is None:
            run(0, maxiter, bool(p.normalize))
        else:
            # checks happen at i % update == 0, after that iteration's update
            i = 0
            while i < maxiter and not stopped.value:
                run(i, 1, False)
                p.callback(g.cpu().numpy(), i, float(mags[nm.value - 1]))
                i += 1
                if stopped.value:
                    break
                cnt = min(update - 1, maxiter - i)
                if cnt > 0:
                    run(i, cnt, False)
                    i += cnt
            if p.normalize:
                run(it.value, 0, True)
        self.last_iterations = int(it.value)
        self.last_mags = np.array(mags[:min(nm.value, cap)], np.float64)
        return g if self._on_device else g.cpu().numpy()
