"""The C-ABI library builds, loads without a GPU and exports every function
declared in include/*.h; argument validation that needs no GPU."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(m16_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from miccai2016_gb300 import _native
    return _native.lib()


def test_header_declares_entry_points():
    names = _declared()
    assert "m16_maxflow_solve" in names and len(names) >= 4


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(lib):
    from miccai2016_gb300 import _native as N
    assert N.status_string(0) == "ok"
    assert "workspace" in N.status_string(N.M16_ERR_WORKSPACE)
    assert lib.m16_abi_version() >= 1


def test_workspace_bytes_grows_with_volume(lib):
    from miccai2016_gb300 import _native as N
    p = N.CutParams(0.2, 0.11, 1e-4, 100, 10, (ctypes.c_double * 3)(1, 1, 1))
    small = lib.m16_maxflow_workspace_bytes(8, 8, 8, ctypes.byref(p))
    big = lib.m16_maxflow_workspace_bytes(64, 64, 64, ctypes.byref(p))
    assert 0 < small < big
    assert big >= 64 ** 3 * 4 * 9
    assert lib.m16_maxflow_workspace_bytes(0, 8, 8, ctypes.byref(p)) == 0


def test_solve_rejects_bad_arguments_before_touching_the_gpu(lib):
    from miccai2016_gb300 import _native as N
    p = N.CutParams(0.2, 0.11, 1e-4, 100, 10, (ctypes.c_double * 3)(1, 1, 1))
    it = ctypes.c_int32(0)
    sq = (ctypes.c_double * 3)(1, 1, 1)
    fake = ctypes.c_void_p(256)
    # zero-sized volume
    st = lib.m16_maxflow_solve(fake, fake, sq, None, None, 0.1, fake, fake, None, 0, 4, 4, ctypes.byref(p), fake,
                               ctypes.byref(it), None, 0, None, fake, 1 << 20, None)
    assert st == N.M16_ERR_BAD_SHAPE
    # update < 1
    p.update = 0
    st = lib.m16_maxflow_solve(fake, fake, sq, None, None, 0.1, fake, fake, None, 4, 4, 4, ctypes.byref(p), fake,
                               ctypes.byref(it), None, 0, None, fake, 1 << 20, None)
    assert st == N.M16_ERR_BAD_ARG
    p.update = 10
    # workspace too small
    st = lib.m16_maxflow_solve(fake, fake, sq, None, None, 0.1, fake, fake, None, 4, 4, 4, ctypes.byref(p), fake,
                               ctypes.byref(it), None, 0, None, fake, 16, None)
    assert st == N.M16_ERR_WORKSPACE
    # neither constant nor per-voxel eigenvalues
    st = lib.m16_maxflow_solve(fake, fake, None, None, None, 0.1, fake, fake, None, 4, 4, 4, ctypes.byref(p), fake,
                               ctypes.byref(it), None, 0, None, fake, 1 << 20, None)
    assert st == N.M16_ERR_BAD_ARG


def test_solve_ex_rejects_an_unknown_iteration_path(lib):
    from miccai2016_gb300 import _native as N
    p = N.CutParams(0.2, 0.11, 1e-4, 100, 10, (ctypes.c_double * 3)(1, 1, 1))
    it = ctypes.c_int32(0)
    sq = (ctypes.c_double * 3)(1, 1, 1)
    fake = ctypes.c_void_p(256)
    for path in (-1, 4):
        s = N.SolveStats(0, 0, 0, 0, 0.0, 0.0, path, 0)
        st = lib.m16_maxflow_solve_ex(fake, fake, sq, None, None, 0.1, fake, fake, None, 4, 4, 4, ctypes.byref(p),
                                      fake, ctypes.byref(it), None, 0, None, fake, 1 << 20, None, ctypes.byref(s))
        assert st == N.M16_ERR_BAD_ARG


def test_server_create_validates_before_touching_the_gpu(lib):
    from miccai2016_gb300 import _native as N
    h = ctypes.c_void_p()
    p = N.CutParams(0.2, 0.11, 1e-4, 100, 30, (ctypes.c_double * 3)(1, 1, 1))   # 100 is not a multiple of 30
    assert lib.m16_server_create(ctypes.byref(p), 4, 1024, ctypes.c_void_p(256), 1 << 30, None,
                                 ctypes.byref(h)) == N.M16_ERR_BAD_ARG
    p.num_iter = 90
    assert lib.m16_server_create(ctypes.byref(p), 4, 1024, None, 1 << 30, None, ctypes.byref(h)) == N.M16_ERR_WORKSPACE
    assert lib.m16_server_create(ctypes.byref(p), 4, 1024, ctypes.c_void_p(256), 16, None,
                                 ctypes.byref(h)) == N.M16_ERR_WORKSPACE
    assert lib.m16_server_create(ctypes.byref(p), 0, 1024, ctypes.c_void_p(256), 1 << 30, None,
                                 ctypes.byref(h)) == N.M16_ERR_BAD_ARG
    assert not h.value


def test_server_sizes(lib):
    # a resident request holds its inputs (28 B), the expanded quaternions
    # (16 B) and six state fields (24 B) per voxel, plus small per-tile parts
    b = lib.m16_server_request_bytes(64, 64, 64, 0)
    assert 68 * 64 ** 3 <= b <= 68 * 64 ** 3 + (1 << 20)
    assert lib.m16_server_request_bytes(0, 64, 64, 0) == 0
    assert lib.m16_server_table_bytes(16, 1024) > 0


def test_indexed_sign_flip_validates_before_touching_the_gpu(lib):
    from miccai2016_gb300 import _native as N
    fake = ctypes.c_void_p(256)
    sc = (ctypes.c_double * 3)(1, 1, 1)
    nb = lib.m16_adjust_nonridge_signs_workspace_bytes(64, 64, 64, 1000)
    assert nb >= 1000 * 16
    assert lib.m16_adjust_nonridge_signs_workspace_bytes(0, 64, 64, 1000) == 0
    assert lib.m16_adjust_nonridge_signs_workspace_bytes(64, 64, 64, 0) == 0
    # far fewer points than voxels -> larger cells, a smaller index
    assert lib.m16_adjust_nonridge_signs_workspace_bytes(64, 64, 64, 10) < nb
    call = lambda d0, R, s, ws, wsb: lib.m16_adjust_nonridge_signs_indexed(fake, d0, 64, 64, fake, fake, R, s, ws,
                                                                           wsb, None)
    assert call(0, 1000, sc, fake, nb) == N.M16_ERR_BAD_SHAPE
    assert call(70000, 1000, sc, fake, nb) == N.M16_ERR_BAD_SHAPE
    assert call(64, 0, sc, fake, nb) == N.M16_ERR_BAD_ARG
    assert call(64, 1000, (ctypes.c_double * 3)(1, 0, 1), fake, nb) == N.M16_ERR_BAD_ARG
    assert call(64, 1000, sc, None, nb) == N.M16_ERR_WORKSPACE
    assert call(64, 1000, sc, fake, nb - 1) == N.M16_ERR_WORKSPACE
    assert call(64, 1000, sc, ctypes.c_void_p(260), nb) == N.M16_ERR_WORKSPACE


def test_capacities_and_dice_validate_before_touching_the_gpu(lib):
    from miccai2016_gb300 import _native as N
    fake = ctypes.c_void_p(256)
    cap = lambda d0, s, eps, cs, g2: lib.m16_capacities(fake, d0, 8, 8, s, eps, cs, None, g2, None)
    assert cap(0, 1.0, 1e-9, fake, None) == N.M16_ERR_BAD_SHAPE
    assert cap(1, 1.0, 1e-9, None, fake) == N.M16_ERR_BAD_SHAPE     # gradient needs 2 voxels per axis
    assert cap(8, 0.0, 1e-9, fake, None) == N.M16_ERR_BAD_ARG
    assert cap(8, 1.0, 0.0, fake, None) == N.M16_ERR_BAD_ARG
    assert lib.m16_capacities(fake, 8, 8, 8, 1.0, 1e-9, None, None, None, None) == N.M16_ERR_BAD_ARG
    nb = lib.m16_fast_dice_workspace_bytes(3)
    assert nb > 0 and lib.m16_fast_dice_workspace_bytes(0) == 0
    ptrs = (ctypes.c_void_p * 3)(256, 512, None)
    out = (ctypes.c_double * 3)()
    assert lib.m16_fast_dice(ptrs, 3, 100, fake, out, fake, nb, None) == N.M16_ERR_BAD_ARG   # a NULL segmentation
    ptrs = (ctypes.c_void_p * 3)(256, 512, 768)
    assert lib.m16_fast_dice(ptrs, 3, 100, fake, out, fake, nb - 1, None) == N.M16_ERR_WORKSPACE
    assert lib.m16_fast_dice(ptrs, 0, 100, fake, out, fake, nb, None) == N.M16_ERR_BAD_ARG


def test_ridge_mst_validates_before_touching_the_gpu(lib):
    from miccai2016_gb300 import _native as N
    fake = ctypes.c_void_p(256)
    dims = (ctypes.c_int32 * 3)(4, 4, 4)
    lo = (ctypes.c_int32 * 3)(0, 0, 0)
    vs = (ctypes.c_double * 3)(1, 1, 1)
    offs = (ctypes.c_int32 * 3)(0, 0, 1)
    nb = lib.m16_ridge_mst_workspace_bytes(10, dims, 1)
    assert nb >= 64 * 4 + 10 * 24
    assert lib.m16_ridge_mst_workspace_bytes(0, dims, 1) == 0
    n = ctypes.c_int64(-1)
    call = lambda R, d, v, r, wsb: lib.m16_ridge_mst_local(fake, R, lo, d, v, offs, 1, r, fake, ctypes.byref(n),
                                                           fake, wsb, None)
    assert call(0, dims, vs, 1.7, nb) == N.M16_ERR_BAD_SHAPE
    assert call(10, (ctypes.c_int32 * 3)(4, 0, 4), vs, 1.7, nb) == N.M16_ERR_BAD_SHAPE
    assert call(10, dims, (ctypes.c_double * 3)(1, -1, 1), 1.7, nb) == N.M16_ERR_BAD_ARG
    assert call(10, dims, vs, 0.0, nb) == N.M16_ERR_BAD_ARG
    assert call(10, dims, vs, 1.7, nb - 1) == N.M16_ERR_WORKSPACE
    assert call(1, dims, vs, 1.7, lib.m16_ridge_mst_workspace_bytes(1, dims, 1)) == N.M16_OK and n.value == 0


def test_label26_validates_before_touching_the_gpu(lib):
    from miccai2016_gb300 import _native as N
    fake = ctypes.c_void_p(256)
    n = ctypes.c_int32(0)
    nb = lib.m16_label26_workspace_bytes(8, 8, 8)
    assert nb >= 512 * 12 and lib.m16_label26_workspace_bytes(0, 8, 8) == 0
    assert lib.m16_label26_workspace_bytes(2048, 2048, 1024) == 0      # beyond 2^31 voxels
    assert lib.m16_label26(fake, 0, 8, 8, fake, ctypes.byref(n), fake, nb, None) == N.M16_ERR_BAD_SHAPE
    assert lib.m16_label26(None, 8, 8, 8, fake, ctypes.byref(n), fake, nb, None) == N.M16_ERR_BAD_ARG
    assert lib.m16_label26(fake, 8, 8, 8, fake, ctypes.byref(n), fake, nb - 1, None) == N.M16_ERR_WORKSPACE
    assert lib.m16_label_workspace_bytes(8, 8, 8) == nb
    for conn in (0, 4, 8, 18):
        assert lib.m16_label(fake, 8, 8, 8, conn, fake, ctypes.byref(n), fake, nb, None) == N.M16_ERR_BAD_ARG


def test_hysteresis_validates_before_touching_the_gpu(lib):
    from miccai2016_gb300 import _native as N
    fake = ctypes.c_void_p(256)
    nb = lib.m16_hysteresis_workspace_bytes(8, 8, 8)
    assert nb == lib.m16_dice_largest_workspace_bytes(8, 8, 8) and lib.m16_hysteresis_workspace_bytes(0, 8, 8) == 0
    assert lib.m16_hysteresis(fake, fake, 8, 0, 8, fake, fake, nb, None) == N.M16_ERR_BAD_SHAPE
    assert lib.m16_hysteresis(fake, None, 8, 8, 8, fake, fake, nb, None) == N.M16_ERR_BAD_ARG
    assert lib.m16_hysteresis(fake, fake, 8, 8, 8, fake, fake, nb - 1, None) == N.M16_ERR_WORKSPACE


def test_dice_largest_validates_before_touching_the_gpu(lib):
    from miccai2016_gb300 import _native as N
    fake = ctypes.c_void_p(256)
    d = ctypes.c_double(0.0)
    nb = lib.m16_dice_largest_workspace_bytes(8, 8, 8)
    assert nb > lib.m16_label_workspace_bytes(8, 8, 8) and lib.m16_dice_largest_workspace_bytes(8, 0, 8) == 0
    assert lib.m16_dice_largest(fake, fake, 0, 8, 8, 0.5, ctypes.byref(d), None, None, fake, nb,
                                None) == N.M16_ERR_BAD_SHAPE
    assert lib.m16_dice_largest(None, fake, 8, 8, 8, 0.5, ctypes.byref(d), None, None, fake, nb,
                                None) == N.M16_ERR_BAD_ARG
    assert lib.m16_dice_largest(fake, fake, 8, 8, 8, 0.5, None, None, None, fake, nb, None) == N.M16_ERR_BAD_ARG
    assert lib.m16_dice_largest(fake, fake, 8, 8, 8, 0.5, ctypes.byref(d), None, None, fake, nb - 1,
                                None) == N.M16_ERR_WORKSPACE


def test_host_tree_helpers(lib):
    """m16_tree_order / m16_compose_signs are host code: they run without a GPU."""
    from miccai2016_gb300 import _native as N
    import numpy as np
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    # forest: 0-1-2, 3-4; root 2
    ea = np.array([0, 1, 3], np.int32)
    eb = np.array([1, 2, 4], np.int32)
    order = np.empty(5, np.int32)
    pred = np.empty(5, np.int32)
    assert lib.m16_tree_order(5, vp(ea), vp(eb), 3, 2, vp(order), vp(pred)) == N.M16_OK
    assert order.tolist() == [2, 1, 0, 3, 4] and pred.tolist() == [1, 2, -1, -1, 3]
    e = np.array([-1, 1, 0, 0, 2], np.int8)
    s = np.zeros(5, np.int8)
    assert lib.m16_compose_signs(5, vp(order), 5, vp(pred), vp(e), vp(s)) == N.M16_OK
    assert s.tolist() == [-1, 1, 1, 1, -1]
    bad = np.array([0, 7], np.int32)
    assert lib.m16_tree_order(5, vp(bad), vp(bad), 2, 0, vp(order), vp(pred)) == N.M16_ERR_BAD_ARG
    assert lib.m16_tree_order(5, vp(ea), vp(eb), 3, 9, vp(order), vp(pred)) == N.M16_ERR_BAD_ARG


def test_batch_steps_validate_before_touching_the_gpu(lib):
    from miccai2016_gb300 import _native as N
    fake = ctypes.c_void_p(256)
    vd = (N.BatchVolume * 1)()
    vd[0] = N.BatchVolume(8, 8, 8, 0, fake, fake, fake, fake, fake, (ctypes.c_double * 3)(1, 1, 1))
    idesc = (N.BatchInstance * 1)()
    idesc[0] = N.BatchInstance(0, 0, 0.1, 3.0, None, (ctypes.c_double * 3)(1, 1, 1), fake)
    p = N.CutParams(0.2, 0.11, 1e-4, 100, 10, (ctypes.c_double * 3)(1, 1, 1))
    h = ctypes.c_void_p()
    nb = lib.m16_batch_workspace_bytes(vd, 1, idesc, 1)
    assert nb > 0
    assert lib.m16_batch_begin(vd, 1, idesc, 1, ctypes.byref(p), fake, nb - 1, None, ctypes.byref(h)) == \
        N.M16_ERR_WORKSPACE and not h.value
    bad = N.CutParams(0.2, 0.11, 1e-4, 100, 0, (ctypes.c_double * 3)(1, 1, 1))   # update 0
    assert lib.m16_batch_begin(vd, 1, idesc, 1, ctypes.byref(bad), fake, nb, None, ctypes.byref(h)) == \
        N.M16_ERR_BAD_ARG
    assert lib.m16_batch_begin(vd, 0, idesc, 1, ctypes.byref(p), fake, nb, None, ctypes.byref(h)) == \
        N.M16_ERR_BAD_ARG
    assert lib.m16_batch_begin(vd, 1, idesc, 1, ctypes.byref(p), fake, nb, None, None) == N.M16_ERR_BAD_ARG
    assert lib.m16_batch_iterate(None, 5, None) == N.M16_ERR_BAD_ARG
    assert lib.m16_batch_end(None, None, None, None) == N.M16_ERR_BAD_ARG
