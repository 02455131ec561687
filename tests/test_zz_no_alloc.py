"""m16_maxflow_solve_static: the max-flow solve for callers that cannot
allocate device memory (a plugin whose host owns all device memory, a
foreign-language binding that needs a fixed footprint, a service that must
not allocate while serving).  It keeps its scratch in a fixed array inside
the library instead of a caller workspace.

Called through the C ABI and checked against m16_maxflow_solve (the
workspace entry point) on calls in a row -- the second with a different
shape and eigenvalue mode, so leftovers of the first call would show.  Both
entry points run the same two-sweep iteration on the same kernels, so u, the
iteration count and every residual must agree bit for bit; each result is
also checked against the CPU oracle within the max-flow tolerance.  After a
warm-up call, a static call must leave the device's free memory unchanged.
Collected last on purpose: if it fails, a run that stops at the first
failure has already run every other test."""
import ctypes
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import inputs as I  # noqa: E402

pytestmark = pytest.mark.gpu

U_TOL = 1e-3          # the tolerance of the max-flow parity tests against the oracle
MAX_VOXELS = 262144   # the documented limit (64 x 64 x 64)
TOO_LARGE = 6         # M16_ERR_TOO_LARGE
CONST_SQ = (1.0, 10 ** -0.75, 10 ** -0.75)


def _lib():
    from miccai2016_gb300 import _native as N
    L = N.lib()
    L.m16_maxflow_solve_static.restype = ctypes.c_int
    L.m16_maxflow_solve_static.argtypes = L.m16_maxflow_solve.argtypes[:18] + [ctypes.c_void_p]
    return N, L


def _case(seed, shape, pointwise, supervised):
    rng = np.random.RandomState(seed)
    img = rng.normal(0.5, 0.5, shape).astype(np.float32)
    q = I.random_squeezed(rng, shape)
    alpha = rng.uniform(0.01, 0.5, shape).astype(np.float32)
    cs = rng.uniform(0, 1, shape).astype(np.float32)
    ct = rng.uniform(0, 1, shape).astype(np.float32)
    sqe = np.sqrt(rng.uniform(0.01, 2, shape + (3,))).astype(np.float32) if pointwise else None
    lab = rng.randint(0, 3, shape).astype(np.uint8) if supervised else None
    return img, q, alpha, cs, ct, sqe, lab


def _solve(N, L, static, case, num_iter=60, update=10):
    """One solve through the C ABI.  Returns (u, iterations, residuals, the
    device's free bytes before and after the call)."""
    import torch
    img, q, alpha, cs, ct, sqe, lab = case
    shape = img.shape
    d = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda()
    dimg, dq, dal, dcs, dct, dsq, dlab = map(d, (img, q, alpha, cs, ct, sqe, lab))
    u = torch.empty(shape, dtype=torch.float32, device="cuda")
    cp = N.CutParams(0.2, 0.11, -1.0, num_iter, update, (ctypes.c_double * 3)(1, 1, 1))
    sq = None if sqe is not None else (ctypes.c_double * 3)(*CONST_SQ)
    it = ctypes.c_int32(0)
    cap = num_iter // update + 2
    res = (ctypes.c_double * cap)()
    nres = ctypes.c_int32(0)
    common = (N.ptr(dimg), N.ptr(dq), sq, N.ptr(dsq), N.ptr(dal), 0.0, N.ptr(dcs), N.ptr(dct), N.ptr(dlab),
              shape[0], shape[1], shape[2], ctypes.byref(cp), N.ptr(u), ctypes.byref(it), res, cap,
              ctypes.byref(nres))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if static:
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st = L.m16_maxflow_solve_static(*common, stream)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
    else:
        nbytes = L.m16_maxflow_workspace_bytes(shape[0], shape[1], shape[2], ctypes.byref(cp))
        ws = N.workspace(nbytes)
        st = L.m16_maxflow_solve(*common, N.ptr(ws), ws.numel(), stream)
        free_before = free_after = None
    assert st == 0, N.status_string(st)
    torch.cuda.synchronize()
    return u.cpu().numpy(), it.value, np.array(res[:nres.value]), free_before, free_after


def _oracle(case, num_iter=60, update=10):
    from oracle import oracle as O
    img, q, alpha, cs, ct, sqe, lab = case
    # the oracle takes eigenvalues and squares back: sqrt(float64(s)^2) == s exactly
    eigs = np.square(sqe.astype(np.float64)) if sqe is not None else np.square(np.array(CONST_SQ))
    u, iters, _ = O.maxflow_solve(img, q, eigs, alpha, cs, ct, labels=lab, num_iter=num_iter, update=update,
                                  error_bound=-1.0)
    return u, iters


def test_static_matches_workspace_entry_point_on_two_calls_in_a_row():
    N, L = _lib()
    cases = [_case(1, (64, 64, 64), pointwise=False, supervised=False),   # the size limit exactly
             _case(2, (17, 9, 33), pointwise=True, supervised=True)]
    first = None
    for case in cases:
        u_s, it_s, r_s, _, _ = _solve(N, L, True, case)
        u_w, it_w, r_w, _, _ = _solve(N, L, False, case)
        assert it_s == it_w == 60
        # the same two-sweep kernels on the same inputs: identical bits
        assert np.array_equal(u_s, u_w)
        assert np.array_equal(r_s, r_w)
        u_o, it_o = _oracle(case)
        assert it_o == 60
        assert np.max(np.abs(u_s - u_o)) <= U_TOL
        if first is None:
            first = u_s
    # a third call on the first case, after the second case left its state in
    # the shared array: the same bits as the first call, and (every kernel and
    # the array already loaded) no change in the device's free memory
    u_s, it_s, _, free_before, free_after = _solve(N, L, True, cases[0])
    assert it_s == 60 and np.array_equal(u_s, first)
    assert free_after == free_before, (free_before, free_after)


def test_static_rejects_requests_beyond_its_scratch():
    N, L = _lib()
    cp = N.CutParams(0.2, 0.11, -1.0, 60, 10, (ctypes.c_double * 3)(1, 1, 1))
    it = ctypes.c_int32(0)
    sq = (ctypes.c_double * 3)(1, 1, 1)
    fake = ctypes.c_void_p(256)
    args = lambda d0, d1, d2: (fake, fake, sq, None, None, 0.1, fake, fake, None, d0, d1, d2, ctypes.byref(cp),
                               fake, ctypes.byref(it), None, 0, None, None)
    assert L.m16_maxflow_solve_static(*args(65, 64, 64)) == TOO_LARGE
    assert L.m16_maxflow_solve_static(*args(1, 1, MAX_VOXELS + 1)) == TOO_LARGE
    cp.num_iter, cp.update = 100000, 1    # 100,002 residual checks > 4,096
    assert L.m16_maxflow_solve_static(*args(8, 8, 8)) == TOO_LARGE
    assert "no-allocation" in N.status_string(TOO_LARGE)
