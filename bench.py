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
         the solve's stream in a second pass over the same solves

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun every rank runs its own replica (the solves are independent).

Other workloads (one JSON line each, not the headline):
  --workload stages128|stages256   every pre-cut pipeline stage, timed per call
  --workload ragged                the ragged batch (4 volume shapes x noise levels)
  --workload plain64|plain128      the headline solve at smaller sizes
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


def _affinity():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1


# host threads available to the process, read before any OpenMP runtime binds
# the main thread to one core (OMP_PROC_BIND=close does after its first
# parallel region)
_HOST_THREADS = _affinity()


def _cpu_threads():
    return _HOST_THREADS


def cpu_baseline(cfg, inp, iters=30):
    """The reference kernels (oracle/_ref, when built here) or the oracle port
    on the host cores: `iters` iterations of the solve, timed, and the
    workload's solves/s that rate gives.  Returns (solves/s, kind, seconds,
    sample)."""
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
    sample = "%d of the %d iterations of one %s solve, timed (%.2f s); solves/s = %d / (%d x that time)" % (
        iters, cfg["num_iter"], "x".join(map(str, cfg["shape"])), dt, iters, cfg["num_iter"])
    return solves, kind, dt, sample


def cpu_whole_solves(count=5):
    """Whole solves of the 64^3 helix workload (300 fixed iterations) with the
    reference kernels or the port on the host cores, timed end to end.
    Returns (solves/s, kind, seconds per solve)."""
    os.environ.setdefault("OMP_NUM_THREADS", str(_cpu_threads()))
    os.environ.setdefault("OMP_PROC_BIND", "close")
    from oracle import oracle as O
    from miccai2016_gb300 import phantom as P
    cfg = P.CONFIG_PLAIN_64
    inp = _inputs(cfg)
    kind = "reference" if O.ref() is not None else "port"
    fn = O.ref_maxflow_solve if kind == "reference" else O.maxflow_solve
    args = (inp["img"], inp["quats"], P.ATV_EIGS, inp["alpha"], inp["cs"], inp["ct"])
    fn(*args, num_iter=cfg["num_iter"], update=30, error_bound=-1.0)   # warm-up
    t0 = time.perf_counter()
    for _ in range(count):
        fn(*args, num_iter=cfg["num_iter"], update=30, error_bound=-1.0)
    dt = (time.perf_counter() - t0) / count
    return 1.0 / dt, kind, dt


def run_reference(args, cfg):
    """The reference's CPU path on the host cores.  Each step runs
    --ref-iters iterations of the workload's solve and is timed as it runs;
    ms_per_step is that observed time, and solves/s follows from the
    iteration rate.  Whole 64^3 x 300-iteration solves are timed beside it."""
    rank, world, _ = _rank_info()
    if rank != 0:
        return
    inp = _inputs(cfg)
    for _ in range(args.warmup):
        cpu_baseline(cfg, inp, iters=args.ref_iters)
    vals, secs = [], []
    kinds = set()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, kind, dt, sample = cpu_baseline(cfg, inp, iters=args.ref_iters)
        vals.append(v)
        secs.append(dt)
        kinds.add(kind)
    total = time.perf_counter() - t0
    value = args.ref_iters * len(secs) / (float(np.sum(secs)) * cfg["num_iter"])
    whole_v, whole_kind, whole_s = cpu_whole_solves()
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * float(np.mean(secs)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": _config(cfg),
            "step": "%d of the workload's %d iterations, timed; value = iterations per second / %d" % (
                args.ref_iters, cfg["num_iter"], cfg["num_iter"]),
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": _cpu_threads(), "kind": kinds.pop(),
                             "sample": sample},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "whole_solves_64cube_300it": {"solves_per_s": whole_v, "s_per_solve": whole_s, "kind": whole_kind,
                                          "cores": _cpu_threads()},
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
    from miccai2016_gb300 import replicas
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
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    if dist:
        ms = replicas.max_over_ranks(ms, device=dev)
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
        e2e_s = replicas.max_over_ranks(e2e_s, device=dev)
    e2e_value = world * e2e_steps / e2e_s
    dice = float(P.fast_dice(out.numpy(), inp["truth"]))

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peak, peak_kind = _peaks()
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
                             "frac": F_BYTES * n / (it_ms * 1e-3) / 1e9 / peak, "bytes_per_voxel": F_BYTES,
                             "note": "events around every launch (no launch overlap)"},
               # the timed solves themselves: launches overlap through
               # programmatic dependent launch, no events in between
               "iteration_in_solve": {"ms": ms_per_step / cfg["num_iter"],
                                      "GB/s": F_BYTES * n / (ms_per_step / cfg["num_iter"] * 1e-3) / 1e9,
                                      "frac": F_BYTES * n / (ms_per_step / cfg["num_iter"] * 1e-3) / 1e9 / peak,
                                      "bytes_per_voxel": F_BYTES}}
    cpu_v, kind, cpu_dt, sample = cpu_baseline(cfg, inp, iters=args.cpu_iters) if rank == 0 else (
        None, None, None, None)
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
    if cfg["name"] == "plain256" and not args.no_batched and world == 1:
        # the default workload at N = 1 also reports the grid search, the ragged batch and serving, each
        # against the plain one-solve-per-call path on the same instances (single-GPU measurements: a
        # multi-GPU run reports the replicated solve only)
        line["batched"] = run_batched_grid()
        line["ragged"] = ragged_batch(args.ragged_step)
        if args.served_requests > 0:
            from miccai2016_gb300.serving import make_payloads, served_vs_plain
            payloads = make_payloads(pool=args.served_pool)
            line["served"] = served_vs_plain(n_requests=args.served_requests, rate=50.0, payloads=payloads,
                                             max_resident=args.served_max_resident or None, check=args.served_check)
            if args.served_saturated > 0:
                line["served"]["saturated"] = served_vs_plain(n_requests=args.served_saturated, rate=None,
                                                              payloads=payloads, seed=1, check=8)
            del payloads
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def _plain_solves(cutter, vol, points, eigs):
    """Every (weighting, decay) point solved one call at a time with
    CmfCutQAnisotropicGpu.execute() on the device-resident volume; alpha =
    w * exp(-|grad I|^2 / decay^2) is computed per call in float32, as the
    batched flow sweep evaluates it.  Returns (u list, iterations, seconds)."""
    import torch
    from miccai2016_gb300 import phantom as P
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    us, its = [], []
    torch.cuda.synchronize()
    e0.record(stream)
    for (w, d) in points:
        a = torch.exp(vol["grad2"] * np.float32(-1.0 / d ** 2)) * np.float32(w)
        us.append(cutter.execute(vol["img"], vol["quats"], eigs, a, vol["cs"], vol["ct"], verbose=False))
        its.append(cutter.last_iterations)
    e1.record(stream)
    torch.cuda.synchronize()
    return us, np.asarray(its, np.int64), e0.elapsed_time(e1) / 1000.0


def _timed_batch(bc, vols, insts, **kw):
    import torch
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    us = bc.solve(vols, insts, **kw)
    e1.record(stream)
    torch.cuda.synchronize()
    return us, bc.last_iterations.copy(), e0.elapsed_time(e1) / 1000.0


def run_batched_grid():
    """The batched grid search of the 128^3 noise-1.5 helix: one
    m16_batch_solve over all 425 ATV (weighting, decay) instances, each
    stopping at residual 1e-4, against all 425 plain one-solve-per-call
    solves of the same instances; then the reference experiment's full loop,
    ATV and TV at every grid point (phantom_experiment.py:350-368), as one
    batch of 850 against 850 plain solves.  Dice is compared instance by
    instance."""
    import torch
    from miccai2016_gb300 import phantom as P, pipeline
    from miccai2016_gb300.batched import BatchedCut
    from miccai2016_gb300.capacities import fast_dice
    from miccai2016_gb300.labeling import dice_largest
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
    insts_tv = [dict(volume=0, weighting=w, decay=d, eigs=P.TV_EIGS) for (w, d) in grid]
    truth_d = torch.from_numpy(truth).cuda()
    n_vox = int(np.prod(cfg["shape"]))
    cp = CmfCutQAnisotropicGpu.CutParameters()
    cp.num_iter, cp.update, cp.error_bound = cfg["num_iter"], cfg["update"], cfg["error_bound"]
    cutter = CmfCutQAnisotropicGpu(cp)
    # warm-up: a two-instance batch and one plain solve load the kernels
    wp = BatchedCut.CutParameters()
    wp.num_iter, wp.update, wp.error_bound = 60, 30, -1.0
    BatchedCut(wp).solve([vol], insts[:2])
    _plain_solves(cutter, vol, grid[:1], P.ATV_EIGS)

    # ---- the 425 ATV instances
    us, iters, batched_s = _timed_batch(bc, [vol], insts)
    tuned_bps = bc.last_blocks_per_sm
    dice_b = np.asarray(fast_dice(us, truth_d))
    best = int(np.argmax(dice_b))
    t_dl = time.perf_counter()
    best_dice_true = dice_largest(us[best], truth_d)
    dice_largest_s = time.perf_counter() - t_dl
    del us
    # the autotuner's candidates, each as a fixed tile shape for the whole
    # solve, and the tuned shape without graph replay
    variants = {}
    for name, kw in (("tile_8_blocks_per_sm", dict(tune=False, blocks_per_sm=8)),
                     ("tile_16_blocks_per_sm", dict(tune=False, blocks_per_sm=16)),
                     ("tile_32_blocks_per_sm", dict(tune=False, blocks_per_sm=32)),
                     ("no_graphs", dict(graphs=False))):
        vu, vit, vs = _timed_batch(bc, [vol], insts, **kw)
        variants[name] = {"s": vs, "blocks_per_sm": bc.last_blocks_per_sm,
                          "same_iterations": bool(np.array_equal(vit, iters))}
        del vu
    plain_u, plain_iters, plain_s = _plain_solves(cutter, vol, grid, P.ATV_EIGS)
    dice_p = np.asarray(fast_dice(plain_u, truth_d))
    plain_best_dice_true = dice_largest(plain_u[best], truth_d)
    del plain_u
    vox_it_b = float(np.sum(iters)) * n_vox
    vox_it_p = float(np.sum(plain_iters)) * n_vox
    atv = {"workload": "425-instance ATV grid search (25 weightings x 17 decays), 128x128x128 helix, "
                       "noise sigma 1.5, stop at residual 1e-4 (update 30, at most 3000 iterations)",
           "solves_per_s": len(insts) / batched_s, "plain_solves_per_s": len(insts) / plain_s,
           "speedup_vs_plain": plain_s / batched_s,
           "plain_sample": "all 425 instances, one CmfCutQAnisotropicGpu.execute() each",
           "batched_s": batched_s, "plain_s": plain_s,
           "iterations": {"min": int(iters.min()), "median": float(np.median(iters)), "max": int(iters.max())},
           "voxel_iterations_per_s": vox_it_b / batched_s, "plain_voxel_iterations_per_s": vox_it_p / plain_s,
           "speedup_voxel_iterations_per_s": (vox_it_b / batched_s) / (vox_it_p / plain_s),
           "achieved_gbs_state": 60.0 * vox_it_b / batched_s / 1e9,   # 60 B of per-instance state per voxel-iteration
           "best_dice_fast": float(dice_b[best]), "best_weighting": grid[best][0], "best_decay": grid[best][1],
           "best_dice_largest_component": best_dice_true, "plain_best_dice_largest_component": plain_best_dice_true,
           "dice_largest_component_s": dice_largest_s,
           "max_dice_diff_vs_plain": float(np.max(np.abs(dice_b - dice_p))),
           "iteration_diff_vs_plain": int(np.max(np.abs(iters - plain_iters))),
           "tuned_blocks_per_sm": tuned_bps, "variants": variants,
           "shared_preparation_s": prep_s, "preparation_stages_s": stages,
           "ridge_points": cut["ridge_points"]}

    # ---- ATV and TV at every grid point, as the reference experiment runs it
    mixed = insts + insts_tv
    us, iters2, batched2_s = _timed_batch(bc, [vol], mixed)
    dice_b2 = np.asarray(fast_dice(us, truth_d))
    del us
    tv_u, tv_iters, tv_s = _plain_solves(cutter, vol, grid, P.TV_EIGS)
    dice_tv = np.asarray(fast_dice(tv_u, truth_d))
    del tv_u
    plain2_s = plain_s + tv_s
    plain2_iters = np.concatenate([plain_iters, tv_iters])
    dice_p2 = np.concatenate([dice_p, dice_tv])
    vox_it_b2 = float(np.sum(iters2)) * n_vox
    vox_it_p2 = float(np.sum(plain2_iters)) * n_vox
    n_atv = len(insts)
    both = {"workload": "850 instances: ATV and TV at each of the 25 x 17 grid points (the reference experiment's "
                        "loop), same volume and stopping rule",
            "solves_per_s": len(mixed) / batched2_s, "plain_solves_per_s": len(mixed) / plain2_s,
            "speedup_vs_plain": plain2_s / batched2_s, "batched_s": batched2_s, "plain_s": plain2_s,
            "voxel_iterations_per_s": vox_it_b2 / batched2_s, "plain_voxel_iterations_per_s": vox_it_p2 / plain2_s,
            "best_dice_fast_atv": float(dice_b2[:n_atv].max()), "best_dice_fast_tv": float(dice_b2[n_atv:].max()),
            "max_dice_diff_vs_plain": float(np.max(np.abs(dice_b2 - dice_p2))),
            "iteration_diff_vs_plain": int(np.max(np.abs(iters2 - plain2_iters)))}
    atv["atv_and_tv"] = both
    return atv


def run_grid_quality(args):
    """Where the grid search's Dice comes from: the 425-instance ATV grid on
    the 128^3 noise-1.5 helix, batched, under each combination of
      * the quaternions: the GPU pipeline's (Frangi, sign adjustment, GVF,
        completion) or the analytic helix tangents;
      * the pipeline's parameters: the workload's (Frangi sigma 2, 4, 6; GVF
        mu 0.2, 100 iterations) or the reference experiment's
        (phantom_experiment.py:228-236, 266-279: Frangi scales
        (r_min / 1.2, r_max * 1.2, 16) for tube radii 3-6, GVF mu 10^0.5,
        300 iterations);
      * the stopping rule: residual 1e-4 (the workload's) or 1e-6 (the
        reference experiment's cutter, phantom_experiment.py:248-256),
        update 30, at most 3000 iterations.
    Prints one JSON line with the best fast Dice, its (weighting, decay) and
    the iteration counts of each combination."""
    import torch
    torch.cuda.set_device(0)
    from miccai2016_gb300 import phantom as P, pipeline
    from miccai2016_gb300.batched import BatchedCut
    from miccai2016_gb300.capacities import fast_dice
    from miccai2016_gb300.labeling import dice_largest
    cfg = P.CONFIG_GRID_128
    nearest = P.helix_nearest(cfg["shape"], cfg["tube_radius"], cfg["helix_radius"], cfg["pitch"])
    noisy, truth = P.helix_phantom(cfg["shape"], cfg["tube_radius"], cfg["helix_radius"], cfg["pitch"],
                                   cfg["sigma"], cfg["seed"], nearest=nearest)
    analytic = P.squeeze_frames(P.helix_tangents(cfg["shape"], cfg["tube_radius"], cfg["helix_radius"],
                                                 cfg["pitch"], nearest=nearest)).astype(np.float32)
    truth_d = torch.from_numpy(truth).cuda()
    preps = {"workload": dict(scales=cfg["scales"], gvf_mu=cfg["gvf_mu"], gvf_iterations=cfg["gvf_iter"]),
             "reference_experiment": dict(scales=(3.0 / 1.2, 6.0 * 1.2, 16), gvf_mu=10 ** 0.5, gvf_iterations=300)}
    grid = [(w, d) for w in cfg["weightings"] for d in cfg["decays"]]
    insts = [dict(volume=0, weighting=w, decay=d, eigs=P.ATV_EIGS) for (w, d) in grid]
    out = {}
    cut0 = None
    for pname, kw in preps.items():
        t0 = time.perf_counter()
        cut, _ = pipeline.prepare_cut_inputs(noisy, cfg["sigma"], **kw)
        prep_s = time.perf_counter() - t0
        cut0 = cut0 or cut
        for qname, quats in (("pipeline", cut["quats"]), ("analytic", analytic)):
            if qname == "analytic" and pname != "workload":
                continue
            for eb in (1e-4, 1e-6):
                bp = BatchedCut.CutParameters()
                bp.num_iter, bp.update, bp.error_bound = 3000, 30, eb
                bc = BatchedCut(bp)
                vol = bc.prepare_volume(noisy, quats, cut["fgw"], cut["bgw"], grad2=cut["grad2"])
                t0 = time.perf_counter()
                us = bc.solve([vol], insts)
                torch.cuda.synchronize()
                solve_s = time.perf_counter() - t0
                dice = np.asarray(fast_dice(us, truth_d))
                best = int(np.argmax(dice))
                out["%s/%s/stop %g" % (qname, pname if qname == "pipeline" else "-", eb)] = {
                    "best_dice_fast": float(dice[best]),
                    "best_dice_largest_component": dice_largest(us[best], truth_d),
                    "best_weighting": grid[best][0], "best_decay": grid[best][1],
                    "iterations_median": float(np.median(bc.last_iterations)),
                    "iterations_at_best": int(bc.last_iterations[best]),
                    "batch_s": solve_s, "preparation_s": prep_s if qname == "pipeline" else None,
                    "ridge_points": cut["ridge_points"] if qname == "pipeline" else None}
                del us
    print(json.dumps({"impl": "ours", "workload": "grid quality: 425 ATV instances, 128^3 helix, noise 1.5",
                      "results": out}), flush=True)


RAGGED_SHAPES = [(96, 96, 96), (128, 128, 192), (160, 160, 160), (224, 224, 160)]


def run_ragged(args):
    """--workload ragged: prints ragged_batch() as one JSON line."""
    import torch
    torch.cuda.set_device(0)
    print(json.dumps(dict(impl="ours", **ragged_batch(args.ragged_step))), flush=True)


def ragged_batch(step=1):
    """Ragged batch: noise levels linspace(0.1, 1.5, 15)[::step] x the four
    volume shapes, each a helix phantom with its own helix radius (0.2-0.3 of
    the smallest extent) and tube radius (2-6 voxels) drawn from a seeded
    RandomState.  Every volume runs the GPU pipeline (Frangi at sigma 1-3,
    sign adjustment, GVF, completion, capacities); then all cuts run as one
    m16_batch_solve (ATV, weighting 10^-1.25, decay 10^1.5, stop at residual
    1e-4, update 30, at most 3000 iterations) against the same cuts solved one
    by one with CmfCutQAnisotropicGpu.execute() on device-resident inputs.
    Returns a dict."""
    import torch
    from miccai2016_gb300 import phantom as P, pipeline
    from miccai2016_gb300.batched import BatchedCut
    from miccai2016_gb300.capacities import fast_dice
    from miccai2016_gb300.continuous_cut_anisotropic_gpu import CmfCutQAnisotropicGpu
    sigmas = np.linspace(0.1, 1.5, 15)[::max(1, step)]
    rng = np.random.RandomState(2016)
    w, d = 10 ** -1.25, 10 ** 1.5
    vols, truths, prep = [], [], []
    bp = BatchedCut.CutParameters()
    bp.num_iter, bp.update, bp.error_bound = 3000, 30, 1e-4
    bc = BatchedCut(bp)
    t_prep = time.perf_counter()
    for sg in sigmas:
        for shape in RAGGED_SHAPES:
            hr = float(rng.uniform(0.2, 0.3) * min(shape))
            tr = float(rng.uniform(2.0, 6.0))
            noisy, truth = P.helix_phantom(shape, tr, hr, 2.5 * hr, float(sg), seed=int(rng.randint(1 << 30)))
            t0 = time.perf_counter()
            cut, _ = pipeline.prepare_cut_inputs(noisy, float(sg), scales=(1, 3, 3))
            prep.append(time.perf_counter() - t0)
            vols.append(bc.prepare_volume(noisy, cut["quats"], cut["fgw"], cut["bgw"], grad2=cut["grad2"]))
            truths.append(torch.from_numpy(truth).cuda())
    t_prep = time.perf_counter() - t_prep
    insts = [dict(volume=k, weighting=w, decay=d, eigs=P.ATV_EIGS) for k in range(len(vols))]
    wp = BatchedCut.CutParameters()
    wp.num_iter, wp.update, wp.error_bound = 60, 30, -1.0
    BatchedCut(wp).solve(vols[:2], insts[:2])   # loads the kernels
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    us = bc.solve(vols, insts)
    e1.record(stream)
    torch.cuda.synchronize()
    batched_s = e0.elapsed_time(e1) / 1000.0
    iters_b = bc.last_iterations.copy()
    dice_b = np.asarray([fast_dice(u, t) for u, t in zip(us, truths)])
    del us
    cp = CmfCutQAnisotropicGpu.CutParameters()
    cp.num_iter, cp.update, cp.error_bound = 3000, 30, 1e-4
    cutter = CmfCutQAnisotropicGpu(cp)
    alphas = [(torch.exp(v["grad2"] * np.float32(-1.0 / d ** 2)) * np.float32(w)).contiguous() for v in vols]
    cutter.execute(vols[0]["img"], vols[0]["quats"], P.ATV_EIGS, alphas[0], vols[0]["cs"], vols[0]["ct"],
                   verbose=False)
    torch.cuda.synchronize()
    plain_s = 0.0
    dice_p, iters_p = [], []
    for v, a, t in zip(vols, alphas, truths):
        e0.record(stream)
        u = cutter.execute(v["img"], v["quats"], P.ATV_EIGS, a, v["cs"], v["ct"], verbose=False)
        e1.record(stream)
        torch.cuda.synchronize()
        plain_s += e0.elapsed_time(e1) / 1000.0
        iters_p.append(cutter.last_iterations)
        dice_p.append(fast_dice(u, t))
    n = len(vols)
    vox = np.array([int(np.prod(v["shape"])) for v in vols], np.float64)
    return {"workload": "ragged batch: %d noise levels x shapes %s, helix phantoms, GPU pipeline "
                                        "per volume, ATV cut w=10^-1.25 decay=10^1.5, stop at residual 1e-4" % (
                                            len(sigmas), RAGGED_SHAPES),
            "volumes": n, "batched_solves_per_s": n / batched_s, "plain_solves_per_s": n / plain_s,
            "speedup_vs_plain": plain_s / batched_s, "batched_s": batched_s, "plain_s": plain_s,
            "voxel_iterations_per_s_batched": float(np.sum(vox * iters_b)) / batched_s,
            "iterations": {"min": int(iters_b.min()), "median": float(np.median(iters_b)), "max": int(iters_b.max())},
            "iteration_diff_vs_plain": int(np.max(np.abs(iters_b - np.asarray(iters_p)))),
            "max_dice_diff_vs_plain": float(np.max(np.abs(dice_b - np.asarray(dice_p)))),
            "dice_fast": {"min": float(dice_b.min()), "median": float(np.median(dice_b)), "max": float(dice_b.max())},
            "preparation_s_per_volume": {"median": float(np.median(prep)), "max": float(np.max(prep))},
            "preparation_total_s": t_prep}


STAGE_BYTES = {
    # algorithmic (compulsory) bytes per unit of each pipeline stage, fp32
    "frangi": 72,          # per voxel-scale: image 4 read, Hessian 24 written + read, val 4 + 4, quat 12
    "detect_ridges": 20,   # per voxel: response 4 + quaternion 12 read, ridge 4 written
    "extract_main_dirs": 24,        # per voxel: quaternion 12 read, direction 12 written
    "detect_ridges_main_dirs": 32,  # both in one pass: response 4 + quaternion 12 read, ridge 4 + direction 12 written
    "gvf": 40,             # per voxel-iteration: g 12, v 12, r 4 read; g 12 written
    "complete_transformations": 24,  # per voxel: direction 12 read, quaternion 12 written
}
STAGES = ["frangi", "detect_ridges", "extract_main_dirs", "detect_ridges_main_dirs", "adjust_nonridge_signs", "gvf",
          "complete_transformations"]


def run_stages(args, cfg):
    """The plain pipeline's stages before the cut, one C-ABI call each on
    device-resident inputs of the workload's helix phantom, timed with CUDA
    events over --steps calls after --warmup calls: Frangi at sigma 1, 2, 3
    (c from the Hessian norm), ridge candidates, main directions, the indexed
    nearest-ridge sign flip (its ridge list from the host steps of
    AdvancedAdjuster), GVF (100 iterations, mu 0.2) and the completion to
    quaternions.  --stages picks a subset (the others run untimed where a
    later stage needs their output).  Prints one JSON line."""
    import contextlib
    import io

    import torch
    torch.cuda.set_device(0)
    from miccai2016_gb300 import _native as N
    from miccai2016_gb300 import phantom as P
    from miccai2016_gb300.adjust_directions import AdvancedAdjuster
    from miccai2016_gb300.gradient_vector_flow import time_step_for
    from miccai2016_gb300.qfrangi_gpu import pack_taps, scales_in_voxels

    L = N.lib()
    shape = tuple(cfg["shape"])
    d0, d1, d2 = shape
    n = d0 * d1 * d2
    noisy, _ = P.helix_phantom(shape, cfg["tube_radius"], cfg["helix_radius"], cfg["pitch"], cfg["sigma"],
                               cfg["seed"])
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream()
    sp = N.stream_ptr()
    peak, peak_kind = _peaks()
    img = torch.from_numpy(noisy).to(dev)
    wanted = set(args.stages.split(",")) if args.stages else set(STAGES)
    unknown = wanted - set(STAGES)
    if unknown:
        raise SystemExit("unknown stages %s" % sorted(unknown))

    def timed(fn, steps=args.steps, warmup=args.warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    out = {}

    def stage(name, fn, units, unit_name, bytes_per_unit=None, extra=None):
        """Times fn when the stage is wanted, else runs it once."""
        if name not in wanted:
            fn()
            return
        ms = timed(fn)
        ent = {"ms": ms, unit_name: units, "units_per_s": units / (ms * 1e-3)}
        if bytes_per_unit is not None:
            gbs = bytes_per_unit * units / (ms * 1e-3) / 1e9
            ent.update({"bytes_per_unit": bytes_per_unit, "GB/s": gbs, "frac": gbs / peak})
        if extra:
            ent.update(extra(ms) if callable(extra) else extra)
        out[name] = ent

    # Frangi, scales 1..3 (3 scales), c = None
    sig = scales_in_voxels((1, 3, 3), np.ones(3))
    taps, radius = pack_taps(sig)
    m = sig.shape[0]
    val = torch.empty(shape, dtype=torch.float32, device=dev)
    quat = torch.empty(shape + (3,), dtype=torch.float32, device=dev)
    ws = N.workspace(L.m16_frangi_workspace_bytes(d0, d1, d2, m))
    stage("frangi", lambda: N.check("m16_frangi", L.m16_frangi(
        N.ptr(img), d0, d1, d2, m, taps.ctypes.data_as(ctypes.c_void_p), radius.ctypes.data_as(ctypes.c_void_p),
        0.5, 0.5, -1.0, 1, N.ptr(val), N.ptr(quat), None, N.ptr(ws), ws.numel(), sp)),
        n * m, "voxel_scales", STAGE_BYTES["frangi"], {"scales": [1, 2, 3], "c": "half the max Hessian norm per scale"})
    del ws
    vmin, vmax = float(val.min()), float(val.max())
    resp = ((val - vmin) / (vmax - vmin)).contiguous()

    ridge = torch.empty(shape, dtype=torch.float32, device=dev)
    stage("detect_ridges", lambda: N.check("m16_detect_ridges", L.m16_detect_ridges(
        N.ptr(resp), N.ptr(quat), d0, d1, d2, 0.01, N.ptr(ridge), sp)), n, "voxels", STAGE_BYTES["detect_ridges"])
    dirs = torch.empty_like(quat)
    stage("extract_main_dirs", lambda: N.check("m16_extract_main_directions", L.m16_extract_main_directions(
        N.ptr(quat), n, N.ptr(dirs), sp)), n, "voxels", STAGE_BYTES["extract_main_dirs"])

    dirs2 = torch.empty_like(quat)
    stage("detect_ridges_main_dirs", lambda: N.check("m16_detect_ridges_main_directions",
                                                     L.m16_detect_ridges_main_directions(
                                                         N.ptr(resp), N.ptr(quat), d0, d1, d2, 0.01, N.ptr(ridge),
                                                         N.ptr(dirs2), sp)),
          n, "voxels", STAGE_BYTES["detect_ridges_main_dirs"])
    del dirs2

    # the ridge list of the host steps (hysteresis, MST, cleaning), then the GPU sign flip
    work = dirs.clone()
    if "adjust_nonridge_signs" in wanted or "gvf" in wanted or "complete_transformations" in wanted:
        q_host, r_host = quat.cpu().numpy(), resp.cpu().numpy()
        for _ in range(2):   # the second run is timed (the first loads kernels and fills caches)
            adj = AdvancedAdjuster(threshold=(0.01, 0.3), qeigs=q_host, response=r_host, voxel_size=(1, 1, 1),
                                   ridge_detection_only=False, clean_ridge=True)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            with contextlib.redirect_stdout(io.StringIO()):
                adj.execute(verbose=False)
            total_s = time.perf_counter() - t0
        adj_timings = dict(adj.timings)
        # the adjuster without its GPU sign flip (timed below as its own stage)
        host_s = total_s - adj_timings.get("nearest_ridge_flip", 0.0)
        coords, rdirs = adj.ridge_coords, adj.ridge_dirs
        R = int(len(coords))
        d_coords = torch.from_numpy(np.ascontiguousarray(coords, np.uint16).view(np.int16)).to(dev)
        d_rdirs = torch.from_numpy(np.ascontiguousarray(rdirs, np.float32)).to(dev)
        sc = (ctypes.c_double * 3)(1.0, 1.0, 1.0)
        nws = N.workspace(L.m16_adjust_nonridge_signs_workspace_bytes(d0, d1, d2, R))
        stage("adjust_nonridge_signs", lambda: N.check("m16_adjust_nonridge_signs_indexed",
                                                       L.m16_adjust_nonridge_signs_indexed(
                                                           N.ptr(work), d0, d1, d2, N.ptr(d_coords), N.ptr(d_rdirs),
                                                           R, sc, N.ptr(nws), nws.numel(), sp)),
              n, "voxels", extra=lambda ms: {
                  "ridge_points": R, "host_steps_s": host_s, "host_steps_breakdown_s": adj_timings,
                  "host_steps": "AdvancedAdjuster.execute() without its nearest-ridge flip: ridge candidates and "
                                "hysteresis, main directions, ridge MST and sign propagation, cleaning",
                  "kernel": "m16_adjust_nonridge_signs_indexed (cell index build + shell search)",
                  "brute_force_equivalent_evaluations_per_s": n * R / (ms * 1e-3)})

    # GVF of the sign-adjusted directions scaled by the response, 100 iterations
    vf = (work * resp.unsqueeze(-1)).contiguous()
    g = torch.empty_like(vf)
    iters = int(cfg.get("gvf_iter", 100))
    mu = float(cfg.get("gvf_mu", 0.2))
    dt = float(time_step_for(np.ones(3), mu, 3))
    cap = iters // 10 + 2
    ws = N.workspace(L.m16_gvf_workspace_bytes(d0, d1, d2, 0, cap))
    vs = (ctypes.c_double * 3)(1.0, 1.0, 1.0)
    mags = (ctypes.c_double * cap)()
    it, stp, nm = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int32(0)
    stage("gvf", lambda: N.check("m16_gvf_run", L.m16_gvf_run(
        N.ptr(vf), None, d0, d1, d2, vs, mu, dt, 0, iters, 10, 0.0, 0, N.ptr(g), ctypes.byref(it),
        ctypes.byref(stp), mags, cap, ctypes.byref(nm), N.ptr(ws), ws.numel(), sp)), n * iters,
        "voxel_iterations", STAGE_BYTES["gvf"], {"iterations": iters, "mu": mu})
    del ws
    q2 = torch.empty_like(g)
    stage("complete_transformations", lambda: N.check("m16_complete_transformations", L.m16_complete_transformations(
        N.ptr(g), n, N.ptr(q2), sp)), n, "voxels", STAGE_BYTES["complete_transformations"])
    line = {"impl": "ours", "workload": "pipeline stages before the cut, %s helix phantom (noise sigma %g)" % (
        "x".join(map(str, shape)), cfg["sigma"]), "steps": args.steps, "warmup": args.warmup,
        "peak_gbs": peak, "peak_kind": peak_kind, "stages": out}
    print(json.dumps(line), flush=True)


def run_paths(args, cfg):
    """The single solve's launches on one workload: the two sweeps with
    programmatic dependent launch (the default) and in plain stream order,
    CUDA events around whole solves and, in a second pass, around every
    launch.  Prints one JSON line."""
    import torch
    torch.cuda.set_device(0)
    from miccai2016_gb300 import _native as N
    from miccai2016_gb300 import phantom as P

    L = N.lib()
    inp = _inputs(cfg)
    shape = cfg["shape"]
    dev = torch.device("cuda", 0)
    d = {k: torch.from_numpy(inp[k]).to(dev) for k in ("img", "quats", "alpha", "cs", "ct")}
    u = torch.empty(shape, dtype=torch.float32, device=dev)
    cp = N.CutParams(0.2, 0.11, -1.0, cfg["num_iter"], 30, (ctypes.c_double * 3)(1, 1, 1))
    ws = N.workspace(L.m16_maxflow_workspace_bytes(shape[0], shape[1], shape[2], ctypes.byref(cp)))
    sq = (ctypes.c_double * 3)(*np.sqrt(P.ATV_EIGS).tolist())
    stream = torch.cuda.current_stream()

    def solve(timing=0, flags=0, path=N.PATH_TWO_SWEEPS):
        s = N.SolveStats(timing, 0, 0, 0, 0.0, 0.0, path, flags)
        it = ctypes.c_int32(0)
        st = L.m16_maxflow_solve_ex(N.ptr(d["img"]), N.ptr(d["quats"]), sq, None, N.ptr(d["alpha"]), 0.0,
                                    N.ptr(d["cs"]), N.ptr(d["ct"]), None, shape[0], shape[1], shape[2],
                                    ctypes.byref(cp), N.ptr(u), ctypes.byref(it), None, 0, None, N.ptr(ws),
                                    ws.numel(), ctypes.c_void_p(stream.cuda_stream), ctypes.byref(s))
        N.check("m16_maxflow_solve_ex", st)
        return s

    def timed(flags=0, path=N.PATH_TWO_SWEEPS):
        for _ in range(args.warmup):
            solve(flags=flags, path=path)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            s = solve(flags=flags, path=path)
        e1.record(stream)
        torch.cuda.synchronize()
        k = solve(timing=1, flags=flags, path=path)
        return dict(ms_per_solve=e0.elapsed_time(e1) / args.steps, launches=s.launches,
                    flow_sweep_ms=k.p_ms / max(k.p_launches, 1), label_sweep_ms=k.u_ms / max(k.u_launches, 1))

    out = {"two_sweeps": timed()}
    u_ref = u.clone()
    out["two_sweeps_no_pdl"] = timed(flags=N.SOLVE_NO_PDL)
    out["two_sweeps_no_pdl"]["max_u_diff_vs_pdl"] = float((u - u_ref).abs().max())
    print(json.dumps({"workload": "launches of one %s solve, %d iterations" % ("x".join(map(str, shape)),
                                                                                cfg["num_iter"]),
                      "steps": args.steps, "warmup": args.warmup, "paths": out}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="plain256")
    ap.add_argument("--ref-iters", type=int, default=30,
                    help="iterations per step of the reference arm and per CPU-baseline sample")
    ap.add_argument("--stages", default="",
                    help="stages workloads: comma-separated subset of %s (default: all)" % ",".join(STAGES))
    ap.add_argument("--ragged-step", type=int, default=1,
                    help="ragged workload: every k-th of the 15 noise levels")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched grid search and the serving comparison of the default workload")
    ap.add_argument("--served-max-resident", type=int, default=0,
                    help="serving comparison: at most this many requests resident at once (0: no limit)")
    ap.add_argument("--served-requests", type=int, default=10000,
                    help="requests of the serving comparison at 50 req/s (0 skips it)")
    ap.add_argument("--served-pool", type=int, default=48,
                    help="serving comparison: distinct helix volumes the requests draw from")
    ap.add_argument("--served-check", type=int, default=32,
                    help="serving comparison: requests whose u is compared between the two loops")
    ap.add_argument("--served-saturated", type=int, default=500,
                    help="serving comparison: requests of the saturated run (all at t = 0; 0 skips it)")
    ap.add_argument("--cpu-iters", type=int, default=100,
                    help="iterations of the CPU-baseline sample of the default arm")
    args = ap.parse_args()
    if args.workload.startswith("paths"):
        run_paths(args, _workload("plain" + args.workload[len("paths"):]))
        return
    if args.workload == "ragged":
        run_ragged(args)
        return
    if args.workload == "grid_quality":
        run_grid_quality(args)
        return
    if args.workload.startswith("stages"):
        run_stages(args, _workload("plain" + args.workload[len("stages"):]))
        return
    cfg = _workload(args.workload)
    if args.impl == "reference":
        run_reference(args, cfg)
    else:
        run_ours(args, cfg)


if __name__ == "__main__":
    main()
