"""
Benchmark of the ATV continuous max-flow on GB300.

Workload (default, "plain256"): the 256^3 float32 helix phantom (tube radius 12,
helix radius 64, pitch 80, noise sigma 1.0, seed 0), ATV eigenvalues
(1, 10^-1.5, 10^-1.5), nonterminal weighting 10^-1.25 and decay 10^1.5,
capacities from the Gaussian log-likelihood ratio, and a fixed 1000 max-flow
iterations (residual checked every 30).  One step = one solve.

  value  solves/s with the inputs resident in HBM (all ranks summed)
  e2e    solves/s through the drop-in CmfCutQAnisotropicGpu.execute() with
         pinned host inputs: H2D of the inputs and D2H of u inside every step
  roofline  the flow sweep (the dominant kernel of an iteration: flow 44 B,
         labels 40 B per voxel), its launch time measured with CUDA events on
         the solve's stream in a second pass over the same solves; the fused
         one-launch iteration (84 B per voxel) is timed once beside it

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun every rank runs its own replica (the solves are independent).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ATV max-flow solves/s batched+served vs plain at equal Dice; p50/p99 latency"
P_BYTES = 44   # flow sweep: tmp 4 + quat 12 + alpha 4 + hp 12 read, hp 12 written
U_BYTES = 40   # label sweep: hp 12 + cs 4 + ct 4 + pt 4 + u 4 read, pt 4 + u 4 + tmp 4 written
F_BYTES = 84   # one iteration (flow + labels), the algorithmic bytes per voxel-iteration


def _rank_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _workload(name):
    from miccai2016_gb300 import phantom as P
    if name == "plain256":
        cfg = dict(P.CONFIG_PLAIN_256)
    elif name == "plain64":
        cfg = dict(P.CONFIG_PLAIN_64)
    elif name == "plain128":
        cfg = dict(P.CONFIG_PLAIN_128)
    else:
        raise SystemExit("unknown workload %s" % name)
    cfg["name"] = name
    return cfg


def _inputs(cfg):
    """Max-flow inputs on the host: image, squeezed quaternions of the helix
    frames, nonterminal weights and capacities (float32)."""
    from miccai2016_gb300 import phantom as P
    noisy, truth, quats, ntw, fgw, bgw = P.maxflow_inputs(cfg)
    return dict(img=noisy, quats=quats, alpha=ntw, cs=fgw, ct=bgw, truth=truth)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic_summary():
    """Per-launch DRAM bytes of the flow/label kernels from the committed ncu
    summary (profiles/maxflow_traffic.json), if present."""
    path = os.path.join(ROOT, "profiles", "maxflow_traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return None


def _cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1


def cpu_baseline(cfg, inp, iters=3):
    """The reference kernels (oracle/_ref, when built here) or the oracle port
    on the host cores: `iters` iterations of the solve, extrapolated to the
    workload's iteration count.  Returns (solves/s, kind, seconds, sample)."""
    os.environ.setdefault("OMP_NUM_THREADS", str(_cpu_threads()))
    os.environ.setdefault("OMP_PROC_BIND", "close")
    from oracle import oracle as O
    from miccai2016_gb300 import phantom as P
    kind = "reference" if O.ref() is not None else "port"
    fn = O.ref_maxflow_solve if kind == "reference" else O.maxflow_solve
    t0 = time.perf_counter()
    fn(inp["img"], inp["quats"], P.ATV_EIGS, inp["alpha"], inp["cs"], inp["ct"], num_iter=iters, update=30,
       error_bound=-1.0)
    dt = time.perf_counter() - t0
    per_iter = dt / iters
    solves = 1.0 / (per_iter * cfg["num_iter"])
    sample = "%d of the %d iterations of one %s solve, extrapolated linearly" % (
        iters, cfg["num_iter"], "x".join(map(str, cfg["shape"])))
    return solves, kind, dt, sample


def run_reference(args, cfg):
    rank, world, _ = _rank_info()
    if rank != 0:
        return
    inp = _inputs(cfg)
    for _ in range(args.warmup):
        cpu_baseline(cfg, inp, iters=1)
    vals = []
    kinds = set()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, kind, dt, sample = cpu_baseline(cfg, inp, iters=args.ref_iters)
        vals.append(v)
        kinds.add(kind)
    total = time.perf_counter() - t0
    value = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": _config(cfg),
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": _cpu_threads(), "kind": kinds.pop(),
                             "sample": sample},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": total}
    print(json.dumps(line), flush=True)


def _config(cfg):
    return {"workload": "ATV max-flow, %s helix phantom, %d fixed iterations" % (
        "x".join(map(str, cfg["shape"])), cfg["num_iter"]),
        "shape": list(cfg["shape"]), "iterations": cfg["num_iter"], "update": 30,
        "eigs": "ATV (1, 10^-1.5, 10^-1.5)", "weighting": cfg["weighting"], "decay": cfg["decay"],
        "noise_sigma": cfg["sigma"], "l2": "inputs+state larger than L2 (no flush needed)"
        if np.prod(cfg["shape"]) * 60 > 129e6 else "working set fits in L2",
        "parallelism": "replicas (one independent solve per GPU)"}


def run_ours(args, cfg):
    import torch
    rank, world, local = _rank_info()
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from miccai2016_gb300 import _native as N
    from miccai2016_gb300 import phantom as P
    from miccai2016_gb300.continuous_cut_anisotropic_gpu import CmfCutQAnisotropicGpu

    L = N.lib()
    inp = _inputs(cfg)
    shape = cfg["shape"]
    n = int(np.prod(shape))
    dev = torch.device("cuda", torch.cuda.current_device())
    d = {k: torch.from_numpy(inp[k]).to(dev) for k in ("img", "quats", "alpha", "cs", "ct")}
    u = torch.empty(shape, dtype=torch.float32, device=dev)
    cp = N.CutParams(0.2, 0.11, -1.0, cfg["num_iter"], 30, (ctypes.c_double * 3)(1, 1, 1))
    nbytes = L.m16_maxflow_workspace_bytes(shape[0], shape[1], shape[2], ctypes.byref(cp))
    ws = N.workspace(nbytes)
    sq = (ctypes.c_double * 3)(*np.sqrt(P.ATV_EIGS).tolist())
    stream = torch.cuda.current_stream()

    def solve(stats=None):
        it = ctypes.c_int32(0)
        st = L.m16_maxflow_solve_ex(N.ptr(d["img"]), N.ptr(d["quats"]), sq, None, N.ptr(d["alpha"]), 0.0,
                                    N.ptr(d["cs"]), N.ptr(d["ct"]), None, shape[0], shape[1], shape[2],
                                    ctypes.byref(cp), N.ptr(u), ctypes.byref(it), None, 0, None, N.ptr(ws),
                                    ws.numel(), ctypes.c_void_p(stream.cuda_stream),
                                    None if stats is None else ctypes.byref(stats))
        N.check("m16_maxflow_solve_ex", st)
        assert it.value == cfg["num_iter"]

    for _ in range(args.warmup):
        solve()
    torch.cuda.synchronize()
    sampler = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    if sampler:
        sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches = 0
    ev0.record(stream)
    for _ in range(args.steps):
        s = N.SolveStats(0, 0, 0, 0, 0.0, 0.0, 0, 0)
        solve(s)
        launches += s.launches
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = ev0.elapsed_time(ev1)
    # the same solves again with every flow / label launch bracketed by CUDA
    # events on the solve's stream: the per-kernel times of the roofline
    p_ms = u_ms = 0.0
    p_n = u_n = 0
    for _ in range(args.steps):
        s = N.SolveStats(1, 0, 0, 0, 0.0, 0.0, N.PATH_DEFAULT, 0)
        solve(s)
        p_ms += s.p_ms; u_ms += s.u_ms; p_n += s.p_launches; u_n += s.u_launches
    # and once with the fused iteration (one launch per iteration) for comparison
    s2 = N.SolveStats(1, 0, 0, 0, 0.0, 0.0, N.PATH_FUSED, 0)
    solve(s2)
    fused_ms, fused_n = s2.p_ms, s2.p_launches
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    if dist:
        t = torch.tensor([ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = world * args.steps / (ms / 1000.0)

    # end to end through the drop-in API with pinned host buffers
    cut_p = CmfCutQAnisotropicGpu.CutParameters()
    cut_p.num_iter, cut_p.update, cut_p.error_bound = cfg["num_iter"], 30, -1.0
    cutter = CmfCutQAnisotropicGpu(cut_p)
    host = {k: torch.from_numpy(inp[k]).pin_memory() for k in ("img", "quats", "alpha", "cs", "ct")}
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    d2h = n * 4
    out = torch.empty(shape, dtype=torch.float32).pin_memory()

    def e2e_step():
        uu = cutter.execute(host["img"], host["quats"], P.ATV_EIGS, host["alpha"], host["cs"], host["ct"],
                            verbose=False)
        out.copy_(uu)

    e2e_step()
    torch.cuda.synchronize()
    e2e_steps = max(1, min(args.steps, 3))
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * e2e_steps / e2e_s
    dice = float(P.fast_dice(out.numpy(), inp["truth"]))

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peak, peak_kind = _peaks()
    f_avg = fused_ms / max(fused_n, 1)
    f_gbs = F_BYTES * n / (f_avg * 1e-3) / 1e9
    p_avg = p_ms / max(p_n, 1)
    u_avg = u_ms / max(u_n, 1)
    p_gbs = P_BYTES * n / (p_avg * 1e-3) / 1e9
    u_gbs = U_BYTES * n / (u_avg * 1e-3) / 1e9
    traffic = _traffic_summary()
    tr = None
    if traffic:
        ent = traffic.get("mf_update_p")
        if ent and ent.get("voxels"):
            tr = float(ent["dram_bytes_per_launch"]) * n / float(ent["voxels"])
    # the dominant kernel of the default (two-sweep) iteration is the flow sweep
    roof = {"bound": "hbm", "kernel": "mf_update_p_kernel (flow sweep of one max-flow iteration)",
            "achieved": p_gbs, "peak": peak, "unit": "GB/s", "frac": p_gbs / peak, "peak_kind": peak_kind,
            "traffic": tr, "algorithmic_bytes_per_launch": P_BYTES * n, "avg_launch_ms": p_avg}
    it_ms = p_avg + u_avg
    kernels = {"mf_update_p": {"avg_ms": p_avg, "launches": p_n, "GB/s": p_gbs, "frac": p_gbs / peak,
                               "bytes_per_voxel": P_BYTES},
               "mf_update_u": {"avg_ms": u_avg, "launches": u_n, "GB/s": u_gbs, "frac": u_gbs / peak,
                               "bytes_per_voxel": U_BYTES},
               "iteration": {"ms": it_ms, "GB/s": F_BYTES * n / (it_ms * 1e-3) / 1e9,
                             "frac": F_BYTES * n / (it_ms * 1e-3) / 1e9 / peak, "bytes_per_voxel": F_BYTES},
               "fused_path": {"mf_fused_kernel_avg_ms": f_avg, "launches": fused_n, "GB/s": f_gbs,
                              "frac": f_gbs / peak, "bytes_per_voxel": F_BYTES}}
    cpu_v, kind, cpu_dt, sample = cpu_baseline(cfg, inp, iters=args.ref_iters)
    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (analytic helix phantom, seeded noise)",
            "config": _config(cfg),
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "steps": e2e_steps},
            "gpu_launches": int(launches), "roofline": roof, "kernels": kernels,
            "cpu_baseline": {"value": cpu_v, "unit": "solves/s", "cores": _cpu_threads(), "kind": kind,
                             "sample": sample},
            "clocks": clocks, "dice_fast": dice,
            "voxel_iterations_per_s": value * n * cfg["num_iter"]}
    if cfg["name"] == "plain256":   # the default workload also reports the batched grid search and serving
        line["batched"] = run_batched_grid()
        if args.served_requests > 0:
            from miccai2016_gb300.serving import served_vs_plain
            line["served"] = served_vs_plain(n_requests=args.served_requests, rate=50.0, pool=8)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_batched_grid(plain_sample=17):
    """The batched grid search (one m16_batch_solve over all 425 ATV
    instances of a 128^3 volume, each stopping at residual 1e-4) against the
    plain one-solve-per-call path on a sample of the same instances."""
    import torch
    from miccai2016_gb300 import phantom as P, pipeline
    from miccai2016_gb300.batched import BatchedCut
    from miccai2016_gb300.continuous_cut_anisotropic_gpu import CmfCutQAnisotropicGpu
    cfg = P.CONFIG_GRID_128
    noisy, truth = P.helix_phantom(cfg["shape"], cfg["tube_radius"], cfg["helix_radius"], cfg["pitch"],
                                   cfg["sigma"], cfg["seed"])
    t0 = time.perf_counter()
    cut, stages = pipeline.prepare_cut_inputs(noisy, cfg["sigma"], scales=cfg["scales"], gvf_mu=cfg["gvf_mu"],
                                              gvf_iterations=cfg["gvf_iter"])
    prep_s = time.perf_counter() - t0
    bp = BatchedCut.CutParameters()
    bp.num_iter, bp.update, bp.error_bound = cfg["num_iter"], cfg["update"], cfg["error_bound"]
    bc = BatchedCut(bp)
    vol = bc.prepare_volume(noisy, cut["quats"], cut["fgw"], cut["bgw"], grad2=cut["grad2"])
    grid = [(w, d) for w in cfg["weightings"] for d in cfg["decays"]]
    insts = [dict(volume=0, weighting=w, decay=d, eigs=P.ATV_EIGS) for (w, d) in grid]
    # warm-up: a two-instance batch loads the kernels
    wp = BatchedCut.CutParameters()
    wp.num_iter, wp.update, wp.error_bound = 60, 30, -1.0
    BatchedCut(wp).solve([vol], insts[:2])
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    us = bc.solve([vol], insts)
    e1.record(stream)
    torch.cuda.synchronize()
    batched_s = e0.elapsed_time(e1) / 1000.0
    iters = bc.last_iterations.copy()
    truth_d = torch.from_numpy(truth).cuda()
    tsum = float(truth_d.sum())
    dice_b = np.array([float(2 * ((u >= 0.5) * truth_d).sum() / ((u >= 0.5).sum() + tsum)) for u in us])
    del us
    best = int(np.argmax(dice_b))
    # plain path on a sample: the decays of the best weighting (17 instances)
    wi = best // len(cfg["decays"])
    sample = [wi * len(cfg["decays"]) + k for k in range(len(cfg["decays"]))][:plain_sample]
    cp = CmfCutQAnisotropicGpu.CutParameters()
    cp.num_iter, cp.update, cp.error_bound = cfg["num_iter"], cfg["update"], cfg["error_bound"]
    cutter = CmfCutQAnisotropicGpu(cp)
    d_img, d_q = vol["img"], vol["quats"]
    alphas = [torch.from_numpy(P.nonterminal_weights(cut["grad2_f64"], grid[k][0], grid[k][1]).astype(np.float32))
              .cuda() for k in sample]
    cutter.execute(d_img, d_q, P.ATV_EIGS, alphas[0], vol["cs"], vol["ct"], verbose=False)   # warm-up
    torch.cuda.synchronize()
    e0.record(stream)
    plain_u = []
    plain_iters = []
    for k, a in zip(sample, alphas):
        plain_u.append(cutter.execute(d_img, d_q, P.ATV_EIGS, a, vol["cs"], vol["ct"], verbose=False))
        plain_iters.append(cutter.last_iterations)
    e1.record(stream)
    torch.cuda.synchronize()
    plain_s = e0.elapsed_time(e1) / 1000.0
    dice_p = np.array([float(2 * ((u >= 0.5) * truth_d).sum() / ((u >= 0.5).sum() + tsum)) for u in plain_u])
    n_vox = int(np.prod(cfg["shape"]))
    vox_it = float(np.sum(iters)) * n_vox
    batched_rate = len(insts) / batched_s
    plain_rate = len(sample) / plain_s
    return {"workload": "425-instance ATV grid search (25 weightings x 17 decays), 128x128x128 helix, "
                        "noise sigma 1.5, stop at residual 1e-4 (update 30, at most 3000 iterations)",
            "solves_per_s": batched_rate, "plain_solves_per_s": plain_rate,
            "speedup_vs_plain": batched_rate / plain_rate,
            "plain_sample": "the 17 decays of the best weighting, one CmfCutQAnisotropicGpu.execute() each",
            "batched_s": batched_s, "plain_sample_s": plain_s,
            "iterations": {"min": int(iters.min()), "median": float(np.median(iters)), "max": int(iters.max())},
            "voxel_iterations_per_s": vox_it / batched_s,
            "achieved_gbs_state": 60.0 * vox_it / batched_s / 1e9,   # flow 28 + label 32 B of state per voxel-iteration
            "best_dice_fast": float(dice_b[best]), "best_weighting": grid[best][0], "best_decay": grid[best][1],
            "max_dice_diff_vs_plain": float(np.max(np.abs(dice_b[sample] - dice_p))),
            "iteration_diff_vs_plain": int(np.max(np.abs(iters[sample] - np.asarray(plain_iters)))),
            "shared_preparation_s": prep_s, "preparation_stages_s": stages,
            "ridge_points": cut["ridge_points"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="plain256")
    ap.add_argument("--ref-iters", type=int, default=3, help="iterations per CPU-baseline sample")
    ap.add_argument("--served-requests", type=int, default=96,
                    help="requests of the serving comparison (0 skips it)")
    args = ap.parse_args()
    cfg = _workload(args.workload)
    if args.impl == "reference":
        run_reference(args, cfg)
    else:
        run_ours(args, cfg)


if __name__ == "__main__":
    main()
