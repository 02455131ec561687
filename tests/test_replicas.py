"""Multi-rank host logic of the replica runs (miccai2016_gb300/replicas.py):
sharding of independent max-flow units, gathering of per-rank results and the
max-over-ranks time, with world_size 2 over gloo on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from miccai2016_gb300 import replicas


def test_shard_covers_every_unit_once():
    for n in (0, 1, 5, 425, 1000):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                seen += replicas.shard(n, r, world)
            assert sorted(seen) == list(range(n))
            counts = replicas.split_counts(n, world)
            assert sum(counts) == n and max(counts) - min(counts) <= (1 if n else 0)


def test_shard_rejects_bad_ranks():
    with pytest.raises(ValueError):
        replicas.shard(10, 2, 2)
    with pytest.raises(ValueError):
        replicas.shard(10, 0, 0)
    with pytest.raises(ValueError):
        replicas.shard(-1, 0, 1)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n_units, drop, out_q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = replicas.shard(n_units, rank, world)
        # a stand-in result per unit: (iterations, dice) as the grid search reports them
        local = {k: (30 * (k + 1), 1.0 / (k + 1)) for k in mine if not (drop and rank == 1 and k == mine[0])}
        t = replicas.max_over_ranks(0.5 + rank)
        try:
            res = replicas.gather_to_root(local, n_units)
            err = None
        except RuntimeError as e:
            res, err = [], str(e)
        out_q.put((rank, mine, t, res, err))
    finally:
        dist.destroy_process_group()


def _run(world, n_units, drop=False):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n_units, drop, q)) for r in range(world)]
    for p in procs:
        p.start()
    outs = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return {o[0]: o[1:] for o in outs}


def test_two_ranks_gather_and_max():
    outs = _run(2, 7)
    assert outs[0][0] == [0, 2, 4, 6] and outs[1][0] == [1, 3, 5]
    assert outs[0][1] == outs[1][1] == 1.5          # the slowest rank's time
    assert outs[0][2] == [(30 * (k + 1), 1.0 / (k + 1)) for k in range(7)]
    assert outs[1][2] == []                         # only rank 0 assembles
    assert outs[0][3] is None


def test_two_ranks_missing_unit_is_an_error():
    outs = _run(2, 6, drop=True)
    assert outs[0][3] is not None and "missing" in outs[0][3]
