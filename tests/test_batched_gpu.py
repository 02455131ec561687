"""The batched engine (csrc/batched.cu) against individual plain solves: every
instance of a batch gives the u of CmfCutQAnisotropicGpu.execute() on the same
inputs within the max-flow tolerance (1e-3 max-abs after a fixed iteration
count; alpha is computed in float on the device instead of float64 on the
host), and stops at the same check."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
U_TOL = 1e-3


def _volume(seed, shape):
    from miccai2016_gb300 import phantom as P
    rng = np.random.RandomState(seed)
    img = rng.normal(0.5, 0.6, shape).astype(np.float32)
    q = np.stack([rng.uniform(-np.pi, np.pi, shape), rng.uniform(0, np.pi, shape),
                  rng.uniform(-np.pi, np.pi, shape)], -1).astype(np.float32)
    bgw, fgw = P.bgfg_weights(img, 0.8)
    grad2 = P.grad_mag_sq(img)
    return dict(img=img, quats=q, cs=fgw.astype(np.float32), ct=bgw.astype(np.float32),
                grad2=grad2.astype(np.float32), grad2_f64=grad2)


def _plain(v, inst, num_iter, update, error_bound):
    from miccai2016_gb300 import phantom as P
    from miccai2016_gb300.continuous_cut_anisotropic_gpu import CmfCutQAnisotropicGpu
    p = CmfCutQAnisotropicGpu.CutParameters()
    p.num_iter, p.update, p.error_bound = num_iter, update, error_bound
    c = CmfCutQAnisotropicGpu(p)
    alpha = inst.get("alpha")
    if alpha is None:
        alpha = P.nonterminal_weights(v["grad2_f64"], inst["weighting"], inst["decay"]).astype(np.float32)
    u = c.execute(v["img"], v["quats"], inst["eigs"], alpha, v["cs"], v["ct"], verbose=False)
    return u, c.last_iterations


def _batch(vols, insts, num_iter, update, error_bound):
    from miccai2016_gb300.batched import BatchedCut
    p = BatchedCut.CutParameters()
    p.num_iter, p.update, p.error_bound = num_iter, update, error_bound
    b = BatchedCut(p)
    dv = [b.prepare_volume(v["img"], v["quats"], v["cs"], v["ct"], grad2=v["grad2"]) for v in vols]
    us = b.solve(dv, insts)
    return [u.cpu().numpy() for u in us], b.last_iterations


ATV = (1.0, 10 ** -1.5, 10 ** -1.5)
TV = (1.0, 1.0, 1.0)


def test_mixed_batch_matches_plain_solves():
    vols = [_volume(1, (24, 20, 36)), _volume(2, (17, 33, 9))]
    insts = [dict(volume=0, weighting=10 ** -1.25, decay=10 ** 1.5, eigs=ATV),
             dict(volume=0, weighting=10 ** -2.0, decay=1.0, eigs=TV),
             dict(volume=1, weighting=0.3, decay=3.0, eigs=ATV),
             dict(volume=0, weighting=0.05, decay=0.5, eigs=ATV),
             dict(volume=1, alpha=np.full((17, 33, 9), 0.07, np.float32), eigs=TV),
             dict(volume=1, weighting=1.0, decay=100.0, eigs=(1.0, 0.5, 0.25))]
    us, its = _batch(vols, insts, 120, 30, -1.0)
    for k, inst in enumerate(insts):
        u, it = _plain(vols[inst["volume"]], inst, 120, 30, -1.0)
        assert its[k] == it == 120
        assert np.max(np.abs(us[k] - u)) <= U_TOL, k


def test_instances_stop_on_their_own():
    vols = [_volume(3, (32, 32, 32))]
    insts = [dict(volume=0, weighting=w, decay=d, eigs=e) for w in (0.01, 0.1, 1.0) for d in (1.0, 30.0)
             for e in (ATV, TV)]
    us, its = _batch(vols, insts, 2000, 10, 2e-3)
    assert len(set(its.tolist())) > 1          # they do not all stop together
    for k, inst in enumerate(insts):
        u, it = _plain(vols[0], inst, 2000, 10, 2e-3)
        assert abs(int(its[k]) - it) <= 10
        if int(its[k]) == it:
            assert np.max(np.abs(us[k] - u)) <= U_TOL


def test_grid_search_shape_of_the_reference():
    """25 x 17 (weighting, decay) points on one volume, as phantom_experiment.py:167-168."""
    vols = [_volume(4, (16, 16, 16))]
    ws = np.logspace(-2.5, 0.5, 25)
    ds = np.logspace(-1, 3, 17)
    insts = [dict(volume=0, weighting=w, decay=d, eigs=ATV) for w in ws for d in ds]
    us, its = _batch(vols, insts, 60, 30, -1.0)
    assert len(us) == 425 and np.all(its == 60)
    for k in (0, 200, 424):
        u, _ = _plain(vols[0], insts[k], 60, 30, -1.0)
        assert np.max(np.abs(us[k] - u)) <= U_TOL


def test_groups_of_four_with_padding_and_mixed_eigenvalues():
    """Instances are grouped four to a group by (volume, eigenvalues, alpha
    kind), interleaved lane by lane; 7 instances of two eigenvalue sets give
    partly filled groups whose padding lanes must not disturb the real ones,
    and an instance alone in its group must match too."""
    vols = [_volume(5, (20, 18, 40))]
    insts = []
    for k in range(7):
        e = ATV if k % 3 else TV
        insts.append(dict(volume=0, weighting=0.02 * (k + 1), decay=0.5 * (k + 1), eigs=e))
    insts.append(dict(volume=0, weighting=0.1, decay=2.0, eigs=(1.0, 0.3, 0.2)))
    us, its = _batch(vols, insts, 90, 30, -1.0)
    for k, inst in enumerate(insts):
        u, it = _plain(vols[0], inst, 90, 30, -1.0)
        assert its[k] == it == 90
        assert np.max(np.abs(us[k] - u)) <= U_TOL, k


def test_graph_replay_equals_direct_launches():
    """Whole check intervals replayed as CUDA graphs (re-captured when
    finished groups leave the work list) give the same bits as launching
    every iteration directly."""
    from miccai2016_gb300.batched import BatchedCut
    vols = [_volume(6, (28, 24, 40)), _volume(7, (16, 16, 16))]
    insts = [dict(volume=v, weighting=w, decay=d, eigs=e) for v in (0, 1) for w in (0.01, 0.1, 1.0)
             for d in (1.0, 30.0) for e in (ATV, TV)]
    p = BatchedCut.CutParameters()
    p.num_iter, p.update, p.error_bound = 1500, 10, 2e-3
    out = []
    for graphs in (True, False):
        b = BatchedCut(p)
        dv = [b.prepare_volume(v["img"], v["quats"], v["cs"], v["ct"], grad2=v["grad2"]) for v in vols]
        us = b.solve(dv, insts, graphs=graphs)
        out.append(([u.cpu().numpy() for u in us], b.last_iterations.copy(), b.last_residuals.copy()))
    (ua, ia, ra), (ub, ib, rb) = out
    assert len(set(ia.tolist())) > 2               # groups finish at different checks
    assert np.array_equal(ia, ib) and np.array_equal(ra, rb, equal_nan=True)
    for a, b_ in zip(ua, ub):
        assert np.array_equal(a.view(np.uint32), b_.view(np.uint32))


def test_tile_shape_tuner_keeps_the_results():
    """The tuner times three tile shapes on the first check intervals of the
    solve itself; the per-voxel arithmetic does not depend on the tile, so
    with a fixed iteration count u is the same bits tuned and untuned, and a
    second batch of the same shape reuses the tuned shape."""
    from miccai2016_gb300.batched import BatchedCut
    vols = [_volume(8, (64, 64, 64))]
    insts = [dict(volume=0, weighting=w, decay=d, eigs=ATV) for w in (0.01, 0.05, 0.2, 1.0) for d in (1.0, 30.0)]
    p = BatchedCut.CutParameters()
    p.num_iter, p.update, p.error_bound = 150, 30, -1.0
    res = []
    for tune in (False, True, True):
        b = BatchedCut(p)
        dv = [b.prepare_volume(v["img"], v["quats"], v["cs"], v["ct"], grad2=v["grad2"]) for v in vols]
        us = b.solve(dv, insts, tune=tune)
        res.append(([u.cpu().numpy() for u in us], b.last_iterations.copy(), b.last_blocks_per_sm))
    assert res[0][2] == 16 and res[1][2] in (8, 16, 32) and res[2][2] == res[1][2]
    for k in range(len(insts)):
        assert res[0][1][k] == res[1][1][k] == 150
        assert np.array_equal(res[0][0][k].view(np.uint32), res[1][0][k].view(np.uint32))
        assert np.array_equal(res[2][0][k].view(np.uint32), res[1][0][k].view(np.uint32))


def test_tuning_graphs_and_a_shrinking_work_list_together():
    """Four-lane groups and a one-lane group in one batch, tuned, replayed as
    graphs, with instances stopping at different checks so the work list
    shrinks while the shape is tuned: every instance still gives its plain
    solve (a graph is never replayed over a work list it was not captured
    from)."""
    from miccai2016_gb300.batched import BatchedCut
    vols = [_volume(9, (48, 48, 48))]
    insts = [dict(volume=0, weighting=w, decay=d, eigs=ATV) for w in (0.003, 0.03, 0.3, 3.0)
             for d in (0.3, 3.0, 30.0)] + [dict(volume=0, weighting=0.05, decay=1.0, eigs=TV)]
    p = BatchedCut.CutParameters()
    p.num_iter, p.update, p.error_bound = 1200, 10, 2e-3
    b = BatchedCut(p)
    dv = [b.prepare_volume(v["img"], v["quats"], v["cs"], v["ct"], grad2=v["grad2"]) for v in vols]
    us = [u.cpu().numpy() for u in b.solve(dv, insts, graphs=True, tune=True)]
    its = b.last_iterations
    assert len(set(its.tolist())) > 2
    for k, inst in enumerate(insts):
        u, it = _plain(vols[0], inst, 1200, 10, 2e-3)
        assert abs(int(its[k]) - it) <= 10
        if int(its[k]) == it:
            assert np.max(np.abs(us[k] - u)) <= U_TOL


def _steps_batch():
    vols = [_volume(21, (30, 26, 40)), _volume(22, (19, 35, 12))]
    insts = [dict(volume=0, weighting=10 ** -1.25, decay=10 ** 1.5, eigs=ATV),
             dict(volume=0, weighting=0.02, decay=3.0, eigs=ATV),
             dict(volume=0, weighting=0.3, decay=0.7, eigs=ATV),
             dict(volume=0, weighting=0.1, decay=30.0, eigs=ATV),      # one four-lane group
             dict(volume=1, weighting=0.05, decay=5.0, eigs=TV),       # one-lane groups
             dict(volume=1, alpha=np.full((19, 35, 12), 0.07, np.float32), eigs=ATV)]
    return vols, insts


def _cut(num_iter, update, error_bound):
    from miccai2016_gb300.batched import BatchedCut
    p = BatchedCut.CutParameters()
    p.num_iter, p.update, p.error_bound = num_iter, update, error_bound
    return BatchedCut(p)


def test_steps_equal_the_whole_solve():
    """m16_batch_begin / iterate (in uneven pieces) / end give the bits and
    iteration counts of m16_batch_solve with the default tile shape."""
    vols, insts = _steps_batch()
    b = _cut(300, 30, 1e-3)
    dv = [b.prepare_volume(v["img"], v["quats"], v["cs"], v["ct"], grad2=v["grad2"]) for v in vols]
    ref = [u.cpu().numpy() for u in b.solve(dv, insts, tune=False, graphs=False)]
    ref_its = b.last_iterations.copy()
    assert ref_its.min() < 300   # some instances stop on their own
    steps = b.begin(dv, insts)
    for count in (7, 23, 45, 1, 100, 200):   # 376 requested: bounded by num_iter
        steps.iterate(count)
    us = [u.cpu().numpy() for u in steps.end()]
    assert np.array_equal(steps.iterations, ref_its)
    for u, r in zip(us, ref):
        assert np.array_equal(u.view(np.uint32), r.view(np.uint32))


def test_steps_replayed_from_a_cuda_graph():
    """One check interval captured into a CUDA graph and replayed gives the
    bits of the direct solve."""
    import torch
    vols, insts = _steps_batch()
    b = _cut(120, 30, -1.0)
    dv = [b.prepare_volume(v["img"], v["quats"], v["cs"], v["ct"], grad2=v["grad2"]) for v in vols]
    ref = [u.cpu().numpy() for u in b.solve(dv, insts, tune=False, graphs=False)]
    steps = b.begin(dv, insts)
    steps.iterate(30)                        # iterations 0..29 directly
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        steps.iterate(30)                    # captured: one interval with its check first
    for _ in range(3):                       # iterations 30..119
        g.replay()
    us = [u.cpu().numpy() for u in steps.end()]
    assert np.all(steps.iterations == 120)
    for u, r in zip(us, ref):
        assert np.array_equal(u.view(np.uint32), r.view(np.uint32))


def _oracle(v, inst, num_iter, update, error_bound):
    from miccai2016_gb300 import phantom as P
    from oracle import oracle as O
    alpha = inst.get("alpha")
    if alpha is None:
        alpha = P.nonterminal_weights(v["grad2_f64"], inst["weighting"], inst["decay"]).astype(np.float32)
    u, it, _ = O.maxflow_solve(v["img"], v["quats"], inst["eigs"], alpha, v["cs"], v["ct"], num_iter=num_iter,
                               update=update, error_bound=error_bound)
    return u, it


def test_batch_instances_match_the_oracle():
    """Each instance of a mixed batch (four-lane groups, a one-lane group, a
    per-voxel alpha, ATV and TV, two volumes) against the CPU oracle
    directly, not only through the plain CUDA path."""
    vols = [_volume(21, (24, 28, 32)), _volume(22, (16, 20, 12))]
    insts = [dict(volume=0, weighting=w, decay=d, eigs=e) for w, d in ((0.05, 30.0), (0.3, 1.0)) for e in (ATV, TV)]
    insts += [dict(volume=0, weighting=0.01, decay=100.0, eigs=ATV),
              dict(volume=1, weighting=0.1, decay=3.0, eigs=(1.0, 0.5, 0.25)),
              dict(volume=1, alpha=np.full((16, 20, 12), 0.07, np.float32), eigs=TV)]
    us, its = _batch(vols, insts, 90, 30, -1.0)
    for k, inst in enumerate(insts):
        u, it = _oracle(vols[inst["volume"]], inst, 90, 30, -1.0)
        assert its[k] == it == 90
        assert np.max(np.abs(us[k] - u)) <= U_TOL, k


def test_batch_stopping_matches_the_oracle():
    """Instances that stop at their own residual check stop where the oracle
    stops (or one check away when the residual sits at the threshold)."""
    vols = [_volume(23, (20, 24, 28))]
    insts = [dict(volume=0, weighting=w, decay=d, eigs=ATV) for w in (0.01, 0.2) for d in (1.0, 30.0)]
    us, its = _batch(vols, insts, 1500, 10, 2e-3)
    same = 0
    for k, inst in enumerate(insts):
        u, it = _oracle(vols[0], inst, 1500, 10, 2e-3)
        assert abs(int(its[k]) - it) <= 10
        if int(its[k]) == it:
            same += 1
            assert np.max(np.abs(us[k] - u)) <= U_TOL, k
    assert same >= len(insts) - 1


def test_fixed_tile_shapes_give_the_same_bits():
    """Each of the autotuner's candidate tile shapes, fixed for the whole
    solve, gives the same u (the tile only changes which block computes a
    voxel; only the residual's partial sums follow the tiling); a shape
    outside the candidates is rejected."""
    import ctypes
    from miccai2016_gb300 import _native as N
    from miccai2016_gb300.batched import BatchedCut
    vols = [_volume(31, (40, 36, 44))]
    insts = [dict(volume=0, weighting=w, decay=d, eigs=ATV) for w in (0.02, 0.2) for d in (1.0, 30.0, 300.0)]
    p = BatchedCut.CutParameters()
    p.num_iter, p.update, p.error_bound = 150, 30, -1.0   # fixed iterations: the residual sums' tiling differs
    b = BatchedCut(p)
    dv = [b.prepare_volume(v["img"], v["quats"], v["cs"], v["ct"], grad2=v["grad2"]) for v in vols]
    out = {}
    for bps in (8, 16, 32):
        us = b.solve(dv, insts, tune=False, blocks_per_sm=bps)
        assert b.last_blocks_per_sm == bps
        out[bps] = ([u.cpu().numpy() for u in us], b.last_iterations.copy())
    for bps in (8, 32):
        assert np.array_equal(out[bps][1], out[16][1])
        for k in range(len(insts)):
            assert np.array_equal(out[bps][0][k], out[16][0][k]), (bps, k)
    with pytest.raises(N.M16Error):
        b.solve(dv, insts, tune=False, blocks_per_sm=12)
