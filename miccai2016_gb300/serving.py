"""
Serving ATV max-flow requests with continuous batching (csrc/serve.cu through
the m16_server_* C ABI), and the plain one-request-at-a-time loop it is
measured against.

A request is one volume (image, squeezed quaternions, |grad I|^2, capacities)
with its (weighting, decay); its result is u.  CutServer admits requests while
its workspace has room, keeps their flow/label state resident, advances all of
them `update` iterations per step and retires each at the residual bound (or
num_iter); a request's result is the same as CmfCutQAnisotropicGpu.execute()
on its inputs alone (the same per-request iteration and check sequence).

run_served() / run_plain() replay one arrival sequence in real time and record
each request's latency (completion minus arrival) -- the reference has no
serving path; the plain loop is its CmfCutQAnisotropicGpu used one request at
a time.
"""
from __future__ import annotations

import ctypes
import time
from collections import deque

import numpy as np

from . import _native as N


class CutServer:
    """Continuous-batching max-flow server over one device workspace."""

    def __init__(self, num_iter=3000, update=30, error_bound=1e-4, cc=0.2, steps=0.11, workspace_bytes=None,
                 max_slots=64, max_work_items=1 << 21):
        torch = N.torch_mod()
        L = N.lib()
        self._L = L
        if workspace_bytes is None:
            free, _ = torch.cuda.mem_get_info()
            workspace_bytes = int(free * 0.8)
        self._ws = N.workspace(int(workspace_bytes))
        self.params = N.CutParams(float(cc), float(steps), float(error_bound), int(num_iter), int(update),
                                  (ctypes.c_double * 3)(1.0, 1.0, 1.0))
        h = ctypes.c_void_p()
        st = L.m16_server_create(ctypes.byref(self.params), int(max_slots), int(max_work_items), N.ptr(self._ws),
                                 self._ws.numel(), N.stream_ptr(), ctypes.byref(h))
        N.check("m16_server_create", st)
        self._h = h
        self._keep = {}   # tag -> the request's host buffers (alive until polled)
        self._cap = int(max_slots)

    @staticmethod
    def request_bytes(shape):
        return int(N.lib().m16_server_request_bytes(int(shape[0]), int(shape[1]), int(shape[2]), 0))

    def admit(self, tag, inputs, weighting, decay, eigs, u_out, scaling=(1.0, 1.0, 1.0)):
        """inputs: dict of host arrays (pinned torch tensors for overlapped
        uploads) img, quats, grad2, cs, ct; u_out: host float32 tensor of the
        volume's shape.  Returns True when admitted."""
        shape = tuple(int(s) for s in inputs["img"].shape)
        sq = np.sqrt(np.asarray(eigs, dtype=np.float64))
        req = N.ServeRequest(shape[0], shape[1], shape[2], 0, _hptr(inputs["img"]), _hptr(inputs["quats"]),
                             _hptr(inputs["grad2"]), None, _hptr(inputs["cs"]), _hptr(inputs["ct"]),
                             (ctypes.c_double * 3)(*scaling), float(weighting), float(decay),
                             (ctypes.c_double * 3)(*sq), _hptr(u_out), int(tag))
        ok = ctypes.c_int32(0)
        N.check("m16_server_admit", self._L.m16_server_admit(self._h, ctypes.byref(req), ctypes.byref(ok)))
        if ok.value:
            self._keep[int(tag)] = (inputs, u_out)
        return bool(ok.value)

    def step(self):
        N.check("m16_server_step", self._L.m16_server_step(self._h))

    def poll(self):
        """[(tag, iterations, residual)] of requests whose u has arrived."""
        tags = (ctypes.c_int64 * self._cap)()
        its = (ctypes.c_int32 * self._cap)()
        res = (ctypes.c_double * self._cap)()
        n = ctypes.c_int32(0)
        N.check("m16_server_poll", self._L.m16_server_poll(self._h, tags, its, res, self._cap, ctypes.byref(n)))
        out = [(int(tags[k]), int(its[k]), float(res[k])) for k in range(n.value)]
        for t, _, _ in out:
            self._keep.pop(t, None)
        return out

    def info(self):
        inf = N.ServerInfo()
        N.check("m16_server_get_info", self._L.m16_server_get_info(self._h, ctypes.byref(inf)))
        return {k: getattr(inf, k) for k, _ in N.ServerInfo._fields_}

    def close(self):
        if self._h:
            N.check("m16_server_destroy", self._L.m16_server_destroy(self._h))
            self._h = None
            self._ws = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _hptr(a):
    if a is None:
        return None
    if N.is_torch(a):
        return a.data_ptr()
    return a.ctypes.data


# ---- synthetic requests -------------------------------------------------------

def helix_request(shape, sigma, seed, device="cuda"):
    """Max-flow inputs of a helix volume of any shape, computed with torch on
    the GPU (the numpy phantom helpers take seconds per 128^3): the helix runs
    along axis 0 with radius 0.25 of the smaller cross-section side, pitch 1.25
    times that, tube radius max(2, radius / 5); noise N(0, sigma) from a
    seeded torch generator.  Returns host pinned float32 tensors img, quats,
    grad2, cs, ct and the truth mask."""
    import torch
    d0, d1, d2 = (int(s) for s in shape)
    R = 0.25 * min(d1, d2)
    r = max(2.0, R / 5.0)
    pitch = 1.25 * R
    f64 = torch.float64
    z = torch.arange(d0, device=device, dtype=f64).view(-1, 1, 1)
    y = torch.arange(d1, device=device, dtype=f64).view(1, -1, 1)
    x = torch.arange(d2, device=device, dtype=f64).view(1, 1, -1)
    zc, yc, xc = (d0 - 1) / 2.0, (d1 - 1) / 2.0, (d2 - 1) / 2.0
    a = pitch / (2 * np.pi)
    tmin = ((r + 1.0) - zc) / a
    tmax = ((d0 - 1) - (r + 1.0) - zc) / a
    dz, dy, dx = (z - zc).expand(d0, d1, d2), (y - yc).expand(d0, d1, d2), (x - xc).expand(d0, d1, d2)
    phi = torch.atan2(dy, dx)
    w = (dz / a - phi) / (2 * np.pi)
    k0 = torch.round(w)
    k1 = k0 + torch.where(w >= k0, 1.0, -1.0)
    best = torch.full_like(dz, float("inf"))
    bt = torch.zeros_like(dz)
    for k in (k0, k1):
        t = phi + 2 * np.pi * k
        for _ in range(4):
            c, s_ = torch.cos(t), torch.sin(t)
            g = -a * dz + a * a * t - R * dy * c + R * dx * s_
            gp = a * a + R * dy * s_ + R * dx * c
            gp = torch.where(gp > 1e-6, gp, torch.full_like(gp, a * a + R * R))
            t = t - torch.clamp(g / gp, -0.5, 0.5)
        t = torch.clamp(t, tmin, tmax)
        dd = (dz - a * t) ** 2 + (dy - R * torch.sin(t)) ** 2 + (dx - R * torch.cos(t)) ** 2
        better = dd < best
        best = torch.where(better, dd, best)
        bt = torch.where(better, t, bt)
    truth = (best.sqrt() <= r).to(f64)
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    noisy = (truth + sigma * torch.randn(truth.shape, generator=gen, device=device, dtype=f64)).float()
    # capacities (phantom.bgfg_weights) and |grad I|^2 (phantom.grad_mag_sq)
    im = noisy.to(f64)
    var = sigma * sigma
    npdf = lambda v, m: torch.exp((v - m) ** 2 * (1 / (-2 * var))) * (1 / np.sqrt(2 * np.pi * var))
    eps = 1e-9
    p_hat = 1 / np.sqrt(2 * np.pi * var)
    lr = torch.log((npdf(im, 1) + eps) / (npdf(im, 0) + eps))
    rq = 1 / np.log((p_hat + eps) / eps)
    bgw, fgw = rq * torch.clamp(-lr, min=0), rq * torch.clamp(lr, min=0)
    grads = torch.gradient(im)
    grad2 = grads[0] ** 2 + grads[1] ** 2 + grads[2] ** 2
    # tangent frames -> squeezed quaternions (phantom.helix_tangents, squeeze_frames)
    v = torch.stack([torch.full_like(bt, a), R * torch.cos(bt), -R * torch.sin(bt)], -1)
    quats = _squeeze_frames_torch(v / v.norm(dim=-1, keepdim=True))
    pin = lambda t: t.float().contiguous().cpu().pin_memory()
    return dict(img=pin(noisy), quats=pin(quats), grad2=pin(grad2), cs=pin(fgw), ct=pin(bgw),
                truth=truth.to(torch.uint8).cpu())


def _squeeze_frames_torch(e0):
    import torch
    zero = torch.zeros_like(e0[..., 0])
    use0 = e0[..., 0].abs() > e0[..., 1].abs()
    e1 = torch.where(use0[..., None], torch.stack([-e0[..., 2], zero, e0[..., 0]], -1),
                     torch.stack([zero, e0[..., 2], -e0[..., 1]], -1))
    e1 = e1 / e1.norm(dim=-1, keepdim=True).clamp_min(1e-300)
    e2 = torch.cross(e0, e1, dim=-1)
    m = torch.stack([e0, e1, e2], -1)
    tr = m[..., 0, 0] + m[..., 1, 1] + m[..., 2, 2]
    w = torch.sqrt(torch.clamp(1 + tr, min=0)) / 2
    x = torch.sqrt(torch.clamp(1 + m[..., 0, 0] - m[..., 1, 1] - m[..., 2, 2], min=0)) / 2
    y = torch.sqrt(torch.clamp(1 - m[..., 0, 0] + m[..., 1, 1] - m[..., 2, 2], min=0)) / 2
    zq = torch.sqrt(torch.clamp(1 - m[..., 0, 0] - m[..., 1, 1] + m[..., 2, 2], min=0)) / 2
    x = torch.copysign(x, m[..., 2, 1] - m[..., 1, 2])
    y = torch.copysign(y, m[..., 0, 2] - m[..., 2, 0])
    zq = torch.copysign(zq, m[..., 1, 0] - m[..., 0, 1])
    phi = torch.atan2(x * zq + y * w, x * w - y * zq)
    theta = torch.acos(torch.clamp(1 - 2 * (x * x + y * y), -1, 1))
    psi = torch.atan2(x * zq - y * w, x * w + y * zq)
    return torch.stack([phi, theta, psi], -1)


GRID_WEIGHTINGS = np.logspace(-2.5, 0.5, 25)
GRID_DECAYS = np.logspace(-1, 3, 17)
ATV_EIGS = (1.0, 10 ** -1.5, 10 ** -1.5)


def make_payloads(pool=16, side_range=(64, 320), sigma_range=(0.1, 1.5), seed=0):
    """`pool` helix volumes: sides uniform in side_range, drawn per axis
    independently; noise sigma uniform in sigma_range."""
    rng = np.random.RandomState(seed)
    payloads = []
    for k in range(pool):
        shape = tuple(int(v) for v in rng.randint(side_range[0], side_range[1] + 1, size=3))
        sigma = float(rng.uniform(*sigma_range))
        p = helix_request(shape, sigma, seed=1000 + k)
        p["sigma"] = sigma
        p["shape"] = shape
        payloads.append(p)
    return payloads


def make_workload(n_requests, rate=50.0, pool=16, side_range=(64, 320), sigma_range=(0.1, 1.5), seed=0,
                  payloads=None):
    """Poisson arrivals at `rate` per second (rate None: all at t = 0); each
    request draws a volume from a pool of `pool` helix volumes (make_payloads,
    or the given payloads) and a (weighting, decay) point of the 25 x 17
    grid.  Returns (payloads, requests) with requests = list of dicts (tag,
    arrival, payload index, weighting, decay)."""
    if payloads is None:
        payloads = make_payloads(pool, side_range, sigma_range, seed)
    pool = len(payloads)
    rng = np.random.RandomState(seed + 7919)
    if rate is None:
        arrivals = np.zeros(n_requests)
    else:
        gaps = rng.exponential(1.0 / rate, size=n_requests)
        arrivals = np.cumsum(gaps) - gaps[0]
    reqs = []
    for t in range(n_requests):
        reqs.append(dict(tag=t, arrival=float(arrivals[t]), payload=int(rng.randint(pool)),
                         weighting=float(GRID_WEIGHTINGS[rng.randint(25)]), decay=float(GRID_DECAYS[rng.randint(17)])))
    return payloads, reqs


def _u_buffer(torch, shape):
    # allocated pinned (from the caching host allocator), not copied into pinned memory
    return torch.empty(shape, dtype=torch.float32, pin_memory=True)


def run_served(server, payloads, requests, max_resident=None, keep=None):
    """Replay the arrivals in real time through the server.  Returns per-tag
    dict of arrival, completion (s from the start), iterations, residual and
    the host u.  With keep set, only requests with tag < keep keep their u;
    the others' pinned buffers go back to the host allocator's cache when they
    finish, so long runs hold a bounded amount of host memory."""
    import torch
    pending = deque(sorted(requests, key=lambda r: r["arrival"]))
    waiting = deque()
    out = {}
    resident = 0     # admitted, not yet handed back
    finished = 0
    t0 = time.perf_counter()
    idle = 0
    while finished < len(requests):
        now = time.perf_counter() - t0
        if not pending and not waiting and resident > 0 and server.info()["resident"] == 0:
            idle += 1   # only downloads left: they end within seconds
            if idle > 200000:
                raise RuntimeError("served requests did not come back")
        while pending and pending[0]["arrival"] <= now:
            waiting.append(pending.popleft())
        while waiting and (max_resident is None or resident < max_resident):
            r = waiting[0]
            p = payloads[r["payload"]]
            u = _u_buffer(torch, p["shape"])
            if not server.admit(r["tag"], p, r["weighting"], r["decay"], ATV_EIGS, u):
                break
            waiting.popleft()
            out[r["tag"]] = dict(arrival=r["arrival"], u=u)
            resident += 1
        if server.info()["resident"] > 0:
            server.step()
        elif resident == 0 and pending:
            time.sleep(max(0.0, min(0.01, pending[0]["arrival"] - (time.perf_counter() - t0))))
        else:
            time.sleep(0.0002)   # only downloads in flight
        for tag, it, res in server.poll():
            out[tag].update(done=time.perf_counter() - t0, iterations=it, residual=res)
            if keep is not None and tag >= keep:
                del out[tag]["u"]
            resident -= 1
            finished += 1
    return out


def run_plain(payloads, requests, num_iter=3000, update=30, error_bound=1e-4, keep=None):
    """The same arrivals served one request at a time by the drop-in
    CmfCutQAnisotropicGpu (inputs from the host, u back to the host).  keep
    as in run_served."""
    import torch
    from .continuous_cut_anisotropic_gpu import CmfCutQAnisotropicGpu
    p = CmfCutQAnisotropicGpu.CutParameters()
    p.num_iter, p.update, p.error_bound = num_iter, update, error_bound
    cutter = CmfCutQAnisotropicGpu(p)
    out = {}
    t0 = time.perf_counter()
    for r in sorted(requests, key=lambda q: q["arrival"]):
        wait = r["arrival"] - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        pl = payloads[r["payload"]]
        dev = {k: pl[k].cuda(non_blocking=True) for k in ("img", "quats", "grad2", "cs", "ct")}
        alpha = r["weighting"] * torch.exp((-1.0 / (r["decay"] ** 2)) * dev["grad2"])
        u = cutter.execute(dev["img"], dev["quats"], ATV_EIGS, alpha, dev["cs"], dev["ct"], verbose=False)
        uh = _u_buffer(torch, pl["shape"])
        uh.copy_(u)
        out[r["tag"]] = dict(arrival=r["arrival"], done=time.perf_counter() - t0,
                             iterations=cutter.last_iterations,
                             residual=float(cutter.last_residuals[-1]) if len(cutter.last_residuals) else float("nan"),
                             u=uh)
        if keep is not None and r["tag"] >= keep:
            del out[r["tag"]]["u"], uh
    return out


def latency_summary(out, voxels=None):
    lat = np.array([v["done"] - v["arrival"] for v in out.values()])
    span = max(v["done"] for v in out.values()) - min(v["arrival"] for v in out.values())
    return dict(requests=len(out), p50_s=float(np.percentile(lat, 50)), p99_s=float(np.percentile(lat, 99)),
                mean_s=float(lat.mean()), solves_per_s=len(out) / span, span_s=span)


def served_vs_plain(n_requests=96, rate=50.0, pool=8, seed=0, max_resident=None, check=4, payloads=None):
    """Both loops on one arrival sequence (rate None: all requests at t = 0,
    the saturated capacity); the first `check` requests' u and iteration
    counts are compared between them."""
    import torch
    payloads, reqs = make_workload(n_requests, rate=rate, pool=pool, seed=seed, payloads=payloads)
    pool = len(payloads)
    # warm both paths on a small request
    warm = [dict(tag=0, arrival=0.0, payload=int(np.argmin([np.prod(p["shape"]) for p in payloads])),
                 weighting=0.05, decay=30.0)]
    srv = CutServer()
    run_served(srv, payloads, warm)
    run_plain(payloads, warm)
    torch.cuda.synchronize()
    info0 = srv.info()
    served = run_served(srv, payloads, reqs, max_resident=max_resident, keep=check)
    info = srv.info()
    gpu_s = (info["gpu_ms"] - info0["gpu_ms"]) / 1000.0
    vox_it = info["voxel_iterations"] - info0["voxel_iterations"]
    srv.close()
    torch.cuda.synchronize()
    plain = run_plain(payloads, reqs, keep=check)
    diffs, itdiff = [], []
    for t in range(min(check, n_requests)):
        diffs.append(float(np.max(np.abs(served[t]["u"].numpy() - plain[t]["u"].numpy()))))
        itdiff.append(abs(served[t]["iterations"] - plain[t]["iterations"]))
    vox = [int(np.prod(payloads[r["payload"]]["shape"])) for r in reqs]
    its = [served[r["tag"]]["iterations"] for r in reqs]
    arrivals = "all at t = 0 (saturated)" if rate is None else "Poisson arrivals at %g/s" % rate
    return dict(workload="%d requests, %s, volumes from a pool of %d helix phantoms with "
                          "sides uniform in 64-320 per axis and noise sigma uniform in 0.1-1.5 (torch-generated "
                          "noise), (weighting, decay) from the 25 x 17 grid, ATV, stop at residual 1e-4 "
                          "(update 30, at most 3000 iterations)" % (n_requests, arrivals, pool),
                checked_requests=min(check, n_requests),
                served=latency_summary(served), plain=latency_summary(plain),
                speedup_solves_per_s=latency_summary(served)["solves_per_s"] / latency_summary(plain)["solves_per_s"],
                mean_voxels=float(np.mean(vox)), iterations={"median": float(np.median(its)), "max": int(max(its))},
                max_u_diff_served_vs_plain=max(diffs) if diffs else None,
                max_iteration_diff_served_vs_plain=max(itdiff) if itdiff else None,
                server_steps=int(info["steps"] - info0["steps"]),
                server_gpu_busy=gpu_s / latency_summary(served)["span_s"],
                server_voxel_iterations_per_gpu_s=vox_it / gpu_s if gpu_s > 0 else None,
                server_gbs_at_84B_per_voxel_iteration=84.0 * vox_it / gpu_s / 1e9 if gpu_s > 0 else None)


def _main(argv=None):
    """python -m miccai2016_gb300.serving --requests 10000 --rate 50"""
    import argparse
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=96)
    ap.add_argument("--rate", type=float, default=50.0)
    ap.add_argument("--pool", type=int, default=8)
    ap.add_argument("--max-resident", type=int, default=None)
    ap.add_argument("--check", type=int, default=4)
    a = ap.parse_args(argv)
    print(json.dumps(served_vs_plain(a.requests, a.rate if a.rate > 0 else None, a.pool, max_resident=a.max_resident,
                                     check=a.check)))


if __name__ == "__main__":
    _main()
