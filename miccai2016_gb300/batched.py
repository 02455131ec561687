"""
Batched ATV max-flow: many CmfCutQAnisotropicGpu solves advanced together in
one launch per sweep (csrc/batched.cu, m16_batch_solve).

The reference's grid search (src/phantom_experiment.py:350-368) calls
CmfCutQAnisotropicGpu.execute() once per (weighting, decay) and cut type with
alpha = weighting * exp(-|grad I|^2 / decay^2) computed on the host.  Here a
batch holds any number of volumes and instances; an instance names its volume,
its (weighting, decay) -- alpha is then computed in the flow sweep from the
volume's |grad I|^2 -- or an explicit alpha field, and its constant
eigenvalues.  Each instance stops on its own at the residual threshold.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N
from .continuous_cut_anisotropic_gpu import CmfCutQAnisotropicGpu


class BatchedCut(object):
    """Batch solver with the cut parameters of CmfCutQAnisotropicGpu.CutParameters."""

    CutParameters = CmfCutQAnisotropicGpu.CutParameters

    def __init__(self, params):
        self.params = params
        self.last_iterations = None
        self.last_residuals = None
        self.last_stats = None
        self._ws = None

    def prepare_volume(self, img, quats, cs, ct, grad2=None, scaling=None):
        """Device copies of one volume's inputs (img, squeezed quaternions,
        capacities and, for (weighting, decay) instances, |grad img|^2)."""
        shape = tuple(int(s) for s in img.shape)
        return dict(shape=shape, img=N.to_device_f32(img, shape), quats=N.to_device_f32(quats, shape + (3,)),
                    cs=N.to_device_f32(cs, shape), ct=N.to_device_f32(ct, shape),
                    grad2=None if grad2 is None else N.to_device_f32(grad2, shape),
                    scaling=(1.0, 1.0, 1.0) if scaling is None else tuple(float(v) for v in scaling))

    def solve(self, volumes, instances, time_kernels=False, path=None, graphs=True, tune=True, blocks_per_sm=0):
        """volumes: list of prepare_volume() dicts; instances: list of dicts
        with 'volume' (index), 'eigs' (3 constant eigenvalues) and either
        ('weighting', 'decay') or 'alpha' (an array of the volume's shape).
        path is accepted for symmetry with the single solve; the batched
        engine has one iteration path (flow and label sweeps over groups of
        four interleaved instances).  graphs=False launches every iteration
        directly instead of replaying CUDA graphs of whole check intervals;
        tune=False keeps the default tile shape instead of timing the
        candidates on the first check intervals, or the shape of
        blocks_per_sm (8, 16 or 32: one of the tuner's candidates);
        last_blocks_per_sm reports the shape in use.
        Returns the list of u (CUDA tensors) in instance order."""
        torch = N.torch_mod()
        L = N.lib()
        nv, ni = len(volumes), len(instances)
        vd = (N.BatchVolume * nv)()
        for k, v in enumerate(volumes):
            d0, d1, d2 = v["shape"]
            vd[k] = N.BatchVolume(d0, d1, d2, 0, N.ptr(v["img"]), N.ptr(v["quats"]), N.ptr(v["grad2"]),
                                  N.ptr(v["cs"]), N.ptr(v["ct"]), (ctypes.c_double * 3)(*v["scaling"]))
        us, keep = [], []
        idesc = (N.BatchInstance * ni)()
        for k, inst in enumerate(instances):
            shape = volumes[inst["volume"]]["shape"]
            u = torch.empty(shape, dtype=torch.float32, device=N.device())
            us.append(u)
            alpha = inst.get("alpha")
            if alpha is not None:
                alpha = N.to_device_f32(alpha, shape)
                keep.append(alpha)
            sq = np.sqrt(np.asarray(inst["eigs"], dtype=np.float64))
            idesc[k] = N.BatchInstance(int(inst["volume"]), 0, float(inst.get("weighting", 0.0)),
                                       float(inst.get("decay", 0.0)), N.ptr(alpha), (ctypes.c_double * 3)(*sq),
                                       N.ptr(u))
        p = self.params
        cp = N.CutParams(float(p.cc), float(p.steps), float(p.error_bound), int(p.num_iter), int(p.update),
                         (ctypes.c_double * 3)(1.0, 1.0, 1.0))
        nbytes = L.m16_batch_workspace_bytes(vd, nv, idesc, ni)
        if nbytes == 0:
            raise ValueError("invalid batch description")
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = None
            self._ws = N.workspace(nbytes)
        iters = (ctypes.c_int32 * ni)()
        res = (ctypes.c_double * ni)()
        stats = N.SolveStats(int(bool(time_kernels)), 0, 0, 0, 0.0, 0.0,
                             N.PATH_DEFAULT if path is None else int(path),
                             (0 if graphs else N.BATCH_NO_GRAPH) | (0 if tune else N.BATCH_NO_TUNE))
        if not tune:
            stats.blocks_per_sm = int(blocks_per_sm)
        st = L.m16_batch_solve(vd, nv, idesc, ni, ctypes.byref(cp), iters, res, N.ptr(self._ws), self._ws.numel(),
                               N.stream_ptr(), ctypes.byref(stats))
        N.check("m16_batch_solve", st)
        self.last_iterations = np.array(iters[:], np.int64)
        self.last_residuals = np.array(res[:], np.float64)
        self.last_stats = stats
        self.last_blocks_per_sm = int(stats.blocks_per_sm)
        return us

    def _describe(self, volumes, instances):
        """ctypes descriptors of a batch, the u outputs and the buffers that
        must stay alive while it runs."""
        torch = N.torch_mod()
        nv, ni = len(volumes), len(instances)
        vd = (N.BatchVolume * nv)()
        for k, v in enumerate(volumes):
            d0, d1, d2 = v["shape"]
            vd[k] = N.BatchVolume(d0, d1, d2, 0, N.ptr(v["img"]), N.ptr(v["quats"]), N.ptr(v["grad2"]),
                                  N.ptr(v["cs"]), N.ptr(v["ct"]), (ctypes.c_double * 3)(*v["scaling"]))
        us, keep = [], []
        idesc = (N.BatchInstance * ni)()
        for k, inst in enumerate(instances):
            shape = volumes[inst["volume"]]["shape"]
            u = torch.empty(shape, dtype=torch.float32, device=N.device())
            us.append(u)
            alpha = inst.get("alpha")
            if alpha is not None:
                alpha = N.to_device_f32(alpha, shape)
                keep.append(alpha)
            sq = np.sqrt(np.asarray(inst["eigs"], dtype=np.float64))
            idesc[k] = N.BatchInstance(int(inst["volume"]), 0, float(inst.get("weighting", 0.0)),
                                       float(inst.get("decay", 0.0)), N.ptr(alpha), (ctypes.c_double * 3)(*sq),
                                       N.ptr(u))
        return vd, idesc, us, keep

    def begin(self, volumes, instances):
        """The batch as capture-safe steps (m16_batch_begin): returns a
        BatchSteps whose iterate(count) only enqueues kernels on the current
        stream (so it may be captured into a CUDA graph) and whose end()
        returns the u of every instance."""
        return BatchSteps(self, volumes, instances)


class BatchSteps(object):
    """m16_batch_begin / m16_batch_iterate / m16_batch_end over one batch."""

    def __init__(self, cut, volumes, instances):
        L = N.lib()
        self._L = L
        self._vd, self._idesc, self._us, self._keep = cut._describe(volumes, instances)
        self._volumes = volumes
        p = cut.params
        self._cp = N.CutParams(float(p.cc), float(p.steps), float(p.error_bound), int(p.num_iter), int(p.update),
                               (ctypes.c_double * 3)(1.0, 1.0, 1.0))
        nbytes = L.m16_batch_workspace_bytes(self._vd, len(volumes), self._idesc, len(instances))
        if nbytes == 0:
            raise ValueError("invalid batch description")
        self._ws = N.workspace(nbytes)
        self._n = len(instances)
        # every (non-capturing) stream the batch's work went to: end() orders
        # itself after all of them, whichever stream is current then
        self._streams = {}
        self._last_stream = None
        self._note_stream()
        h = ctypes.c_void_p()
        N.check("m16_batch_begin", L.m16_batch_begin(self._vd, len(volumes), self._idesc, self._n,
                                                     ctypes.byref(self._cp), N.ptr(self._ws), self._ws.numel(),
                                                     N.stream_ptr(), ctypes.byref(h)))
        self._h = h
        self.iterations = None
        self.residuals = None

    def _note_stream(self):
        torch = N.torch_mod()
        if torch.cuda.is_current_stream_capturing():
            return   # captured work runs wherever the graph is replayed, which the caller orders
        s = torch.cuda.current_stream()
        self._streams[s.cuda_stream] = s
        self._last_stream = s

    def iterate(self, count):
        """Enqueue count iterations on the current stream (capturable)."""
        self._note_stream()
        N.check("m16_batch_iterate", self._L.m16_batch_iterate(self._h, int(count), N.stream_ptr()))

    def end(self):
        """u of every instance (CUDA tensors, instance order); sets
        .iterations and .residuals.  Runs on the current stream after the
        work that begin() and iterate() enqueued on any other stream."""
        if self._h is None:
            raise RuntimeError("the batch has ended")
        cur = N.torch_mod().cuda.current_stream()
        for s in self._streams.values():
            if s.cuda_stream != cur.cuda_stream:
                cur.wait_stream(s)
        its = (ctypes.c_int32 * self._n)()
        res = (ctypes.c_double * self._n)()
        h, self._h = self._h, None
        N.check("m16_batch_end", self._L.m16_batch_end(h, its, res, N.stream_ptr()))
        self.iterations = np.array(its[:], np.int64)
        self.residuals = np.array(res[:], np.float64)
        return self._us

    def __del__(self):
        # a batch dropped without end(): finish it (m16_batch_end waits for
        # its work) before the workspace goes back to the allocator.  It runs
        # on the last stream the batch used, after the others' work.
        try:
            if getattr(self, "_h", None) is not None:
                h, self._h = self._h, None
                last = self._last_stream
                for s in self._streams.values():
                    if s.cuda_stream != last.cuda_stream:
                        last.wait_stream(s)
                self._L.m16_batch_end(h, None, None, ctypes.c_void_p(last.cuda_stream))
        except Exception:
            pass


def _main(argv=None):
    """Timing of one batch: python -m miccai2016_gb300.batched --side 128 --instances 64
    Prints one JSON line with the batch's solves/s and the per-launch device
    time of the batched flow and label sweeps (CUDA events)."""
    import argparse
    import json
    import time

    import torch

    from . import phantom as P
    ap = argparse.ArgumentParser()
    ap.add_argument("--side", type=int, default=128)
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--iters", type=int, default=60)
    ap.add_argument("--time-kernels", action="store_true")
    ap.add_argument("--no-graphs", action="store_true")
    a = ap.parse_args(argv)
    shape = (a.side,) * 3
    s = a.side / 128.0
    noisy, truth, quats, ntw, fgw, bgw = P.maxflow_inputs(dict(shape=shape, tube_radius=6 * s, helix_radius=32 * s,
                                                               pitch=40 * s, sigma=1.5, seed=0, weighting=0.05,
                                                               decay=30.0))
    grad2 = P.grad_mag_sq(noisy).astype(np.float32)
    p = BatchedCut.CutParameters()
    p.num_iter, p.update, p.error_bound = a.iters, 30, -1.0
    bc = BatchedCut(p)
    vol = bc.prepare_volume(noisy, quats, fgw, bgw, grad2=grad2)
    ws = np.logspace(-2.5, 0.5, 25)
    ds = np.logspace(-1, 3, 17)
    insts = [dict(volume=0, weighting=ws[k % 25], decay=ds[k % 17], eigs=P.ATV_EIGS) for k in range(a.instances)]
    bc.solve([vol], insts[:1])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bc.solve([vol], insts, time_kernels=a.time_kernels, graphs=not a.no_graphs)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    st = bc.last_stats
    n = int(np.prod(shape))
    out = dict(side=a.side, instances=a.instances, iters=a.iters, graphs=not a.no_graphs, wall_s=dt,
               voxel_iterations_per_s=a.instances * a.iters * n / dt)
    if a.time_kernels and st.p_launches:
        pm = (st.p_ms + st.u_ms) / st.p_launches
        # state bytes per instance and voxel-iteration: the flow sweep reads
        # tmp 4 + hp 12 and writes hp 12, the label sweep reads hp 12 + pt 4 +
        # u 4 and writes pt 4 + u 4 + tmp 4 = 60 B.  The volume's shared fields
        # (read once per group of four) are not counted.
        sb = 60.0
        out.update(iteration_ms=pm, state_bytes=sb, state_gbs=sb * a.instances * n / (pm * 1e-3) / 1e9)
        if st.u_launches:
            out.update(flow_ms=st.p_ms / st.p_launches, label_ms=st.u_ms / st.u_launches)
    print(json.dumps(out))


if __name__ == "__main__":
    _main()
