"""
Multi-GPU runs of independent max-flow units (solves, grid-search instances,
volumes): one process per GPU, the units dealt out round-robin, no data-path
collective.  The reference is single-device (one OpenCL queue per loader,
src/helpers/cl_helpers.py:105-131); its grid search is a loop over
independent (weighting, decay) points (src/phantom_experiment.py:350-368), so
the only exchanges are the ones below: the per-rank results gathered to rank 0
and the slowest rank's time.

Works with any torch.distributed backend (nccl on GPUs, gloo on CPUs).
"""
from __future__ import annotations

from typing import Dict, List, Sequence


def shard(n_units: int, rank: int, world: int) -> List[int]:
    """Unit indices of `rank`: rank, rank + world, ... (every unit exactly once
    over the ranks; the ranks' counts differ by at most one)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    if n_units < 0:
        raise ValueError("negative unit count")
    return list(range(rank, n_units, world))


def gather_to_root(local: Dict[int, object], n_units: int, group=None) -> List[object]:
    """Rank 0 receives every rank's {unit index: result} and returns the
    results in unit order; other ranks return [].  Raises if a unit is
    missing or reported twice."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    parts = [None] * world if rank == 0 else None
    dist.gather_object(dict(local), parts, dst=0, group=group)
    if rank != 0:
        return []
    merged: Dict[int, object] = {}
    for p in parts:
        for k, v in p.items():
            if k in merged:
                raise RuntimeError("unit %d reported by two ranks" % k)
            merged[int(k)] = v
    missing = [k for k in range(n_units) if k not in merged]
    if missing:
        raise RuntimeError("units %s missing from the gathered results" % missing[:8])
    return [merged[k] for k in range(n_units)]


def max_over_ranks(value: float, group=None, device=None) -> float:
    """The largest `value` over the ranks (the whole job's time is the slowest
    rank's)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def split_counts(n_units: int, world: int) -> Sequence[int]:
    """How many units each rank gets from shard()."""
    return [len(range(r, n_units, world)) for r in range(world)]
