"""
Loader of the CUDA library (include/miccai2016_gb300.h) and the small amount of
glue every drop-in module shares: status checking, device buffers (torch is
used for allocation only), streams and host<->device conversion.

There is no CPU fallback: if the library or a CUDA device is missing, the
calls raise.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import build as _build

M16_OK = 0
M16_ERR_BAD_SHAPE = 1
M16_ERR_BAD_ARG = 2
M16_ERR_WORKSPACE = 3
M16_ERR_CUDA = 4
M16_ERR_TIMEOUT = 5
M16_ERR_TOO_LARGE = 6

_lock = threading.Lock()
_lib = None

_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_f32 = ctypes.c_float
_f64 = ctypes.c_double
_sz = ctypes.c_size_t


class M16Error(RuntimeError):
    """A non-zero status returned by the CUDA library."""

    def __init__(self, fn, status):
        self.status = status
        msg = "%s failed: %s (status %d)" % (fn, status_string(status), status)
        super().__init__(msg)


class CutParams(ctypes.Structure):
    """m16_cut_params (include/miccai2016_gb300.h)."""
    _fields_ = [("cc", _f64), ("steps", _f64), ("error_bound", _f64), ("num_iter", _i32),
                ("update", _i32), ("scaling", _f64 * 3)]


# iteration paths of the single solve (m16_solve_stats.path): both the two sweeps
PATH_DEFAULT, PATH_TWO_SWEEPS = 0, 1


BATCH_NO_GRAPH = 1   # m16_solve_stats.flags
BATCH_NO_TUNE = 2
SOLVE_NO_PDL = 4    # m16_solve_stats.flags: the single solve without programmatic dependent launch


class SolveStats(ctypes.Structure):
    """m16_solve_stats (include/miccai2016_gb300.h)."""
    _fields_ = [("time_kernels", _i32), ("launches", _i32), ("p_launches", _i32), ("u_launches", _i32),
                ("p_ms", _f64), ("u_ms", _f64), ("path", _i32), ("flags", _i32),
                ("blocks_per_sm", _i32), ("pair_launches", _i32), ("pair_ms", _f64), ("pair_zc", _i32),
                ("reserved", _i32)]


class BatchVolume(ctypes.Structure):
    """m16_batch_volume (include/miccai2016_gb300.h)."""
    _fields_ = [("d0", _i32), ("d1", _i32), ("d2", _i32), ("reserved", _i32), ("img", _vp), ("quat3", _vp),
                ("grad2", _vp), ("cs", _vp), ("ct", _vp), ("scaling", _f64 * 3)]


class BatchInstance(ctypes.Structure):
    """m16_batch_instance (include/miccai2016_gb300.h)."""
    _fields_ = [("volume", _i32), ("reserved", _i32), ("weighting", _f64), ("decay", _f64), ("alpha", _vp),
                ("sqevals", _f64 * 3), ("u", _vp)]


class ServeRequest(ctypes.Structure):
    """m16_serve_request (include/miccai2016_gb300.h)."""
    _fields_ = [("d0", _i32), ("d1", _i32), ("d2", _i32), ("reserved", _i32), ("img", _vp), ("quat3", _vp),
                ("grad2", _vp), ("alpha", _vp), ("cs", _vp), ("ct", _vp), ("scaling", _f64 * 3),
                ("weighting", _f64), ("decay", _f64), ("sqevals", _f64 * 3), ("u", _vp), ("tag", _i64)]


class ServerInfo(ctypes.Structure):
    """m16_server_info (include/miccai2016_gb300.h)."""
    _fields_ = [("resident", _i32), ("draining", _i32), ("free_slots", _i32), ("reserved", _i32),
                ("free_bytes", _i64), ("largest_free", _i64), ("steps", _i64), ("voxel_iterations", _i64),
                ("gpu_ms", _f64)]


def _declare(L):
    L.m16_status_string.restype = ctypes.c_char_p
    L.m16_status_string.argtypes = [ctypes.c_int]
    L.m16_abi_version.restype = ctypes.c_int
    L.m16_abi_version.argtypes = []
    L.m16_maxflow_workspace_bytes.restype = _sz
    L.m16_maxflow_workspace_bytes.argtypes = [_i32, _i32, _i32, ctypes.POINTER(CutParams)]
    L.m16_maxflow_solve.restype = ctypes.c_int
    L.m16_maxflow_solve.argtypes = [_vp, _vp, _vp, _vp, _vp, _f32, _vp, _vp, _vp, _i32, _i32, _i32,
                                    ctypes.POINTER(CutParams), _vp, ctypes.POINTER(_i32), _vp, _i32,
                                    ctypes.POINTER(_i32), _vp, _sz, _vp]
    L.m16_maxflow_solve_ex.restype = ctypes.c_int
    L.m16_maxflow_solve_ex.argtypes = L.m16_maxflow_solve.argtypes + [ctypes.POINTER(SolveStats)]
    L.m16_frangi_workspace_bytes.restype = _sz
    L.m16_frangi_workspace_bytes.argtypes = [_i32, _i32, _i32, _i32]
    L.m16_frangi.restype = ctypes.c_int
    L.m16_frangi.argtypes = [_vp, _i32, _i32, _i32, _i32, _vp, _vp, _f32, _f32, _f32, _i32, _vp, _vp, _vp, _vp,
                             _sz, _vp]
    L.m16_hessian.restype = ctypes.c_int
    L.m16_hessian.argtypes = [_vp, _i32, _i32, _i32, _vp, _vp, _vp, _vp, _sz, _vp]
    L.m16_eigs.restype = ctypes.c_int
    L.m16_eigs.argtypes = [_vp, _i64, _vp, _vp]
    L.m16_detect_ridges.restype = ctypes.c_int
    L.m16_detect_ridges.argtypes = [_vp, _vp, _i32, _i32, _i32, _f64, _vp, _vp]
    L.m16_detect_ridges_main_directions.restype = ctypes.c_int
    L.m16_detect_ridges_main_directions.argtypes = [_vp, _vp, _i32, _i32, _i32, _f64, _vp, _vp, _vp]
    L.m16_extract_main_directions.restype = ctypes.c_int
    L.m16_extract_main_directions.argtypes = [_vp, _i64, _vp, _vp]
    L.m16_complete_transformations.restype = ctypes.c_int
    L.m16_complete_transformations.argtypes = [_vp, _i64, _vp, _vp]
    L.m16_adjust_nonridge_signs.restype = ctypes.c_int
    L.m16_adjust_nonridge_signs.argtypes = [_vp, _i32, _i32, _i32, _vp, _vp, _i64, _vp, _vp]
    L.m16_tree_order.restype = ctypes.c_int
    L.m16_tree_order.argtypes = [_i64, _vp, _vp, _i64, _i32, _vp, _vp]
    L.m16_compose_signs.restype = ctypes.c_int
    L.m16_compose_signs.argtypes = [_i64, _vp, _i64, _vp, _vp, _vp]
    L.m16_segment_direction_sums.restype = ctypes.c_int
    L.m16_segment_direction_sums.argtypes = [_vp, _vp, _i64, _vp, _i32, _vp]
    L.m16_ridge_edge_codes.restype = ctypes.c_int
    L.m16_ridge_edge_codes.argtypes = [_vp, _i64, _vp, _vp, _i64, _vp, _vp]
    L.m16_ridge_signs_workspace_bytes.restype = ctypes.c_size_t
    L.m16_ridge_signs_workspace_bytes.argtypes = [_i64, _i64]
    L.m16_ridge_forest_joins_workspace_bytes.restype = ctypes.c_size_t
    L.m16_ridge_forest_joins_workspace_bytes.argtypes = [_i64]
    L.m16_ridge_forest_joins.restype = ctypes.c_int
    L.m16_ridge_forest_joins.argtypes = [_vp, _i64, _vp, _vp, _i64, _i64, _vp, _vp, _vp, _vp, ctypes.c_size_t, _vp]
    L.m16_ridge_signs.restype = ctypes.c_int
    L.m16_ridge_signs.argtypes = [_i64, _vp, _vp, _vp, _i64, _vp, _vp, ctypes.c_size_t, _vp]
    L.m16_label26_workspace_bytes.restype = _sz
    L.m16_label26_workspace_bytes.argtypes = [_i32, _i32, _i32]
    L.m16_label26.restype = ctypes.c_int
    L.m16_label26.argtypes = [_vp, _i32, _i32, _i32, _vp, ctypes.POINTER(_i32), _vp, _sz, _vp]
    L.m16_label_workspace_bytes.restype = _sz
    L.m16_label_workspace_bytes.argtypes = [_i32, _i32, _i32]
    L.m16_label.restype = ctypes.c_int
    L.m16_label.argtypes = [_vp, _i32, _i32, _i32, _i32, _vp, ctypes.POINTER(_i32), _vp, _sz, _vp]
    L.m16_hysteresis_workspace_bytes.restype = _sz
    L.m16_hysteresis_workspace_bytes.argtypes = [_i32, _i32, _i32]
    L.m16_hysteresis.restype = ctypes.c_int
    L.m16_hysteresis.argtypes = [_vp, _vp, _i32, _i32, _i32, _vp, _vp, _sz, _vp]
    L.m16_dice_largest_workspace_bytes.restype = _sz
    L.m16_dice_largest_workspace_bytes.argtypes = [_i32, _i32, _i32]
    L.m16_dice_largest.restype = ctypes.c_int
    L.m16_dice_largest.argtypes = [_vp, _vp, _i32, _i32, _i32, ctypes.c_float, ctypes.POINTER(_f64),
                                   ctypes.POINTER(_i64), ctypes.POINTER(_i32), _vp, _sz, _vp]
    L.m16_ridge_mst_workspace_bytes.restype = _sz
    L.m16_ridge_mst_workspace_bytes.argtypes = [_i64, _vp, _i32]
    L.m16_ridge_mst_local.restype = ctypes.c_int
    L.m16_ridge_mst_local.argtypes = [_vp, _i64, _vp, _vp, _vp, _vp, _i32, _f64, _vp, ctypes.POINTER(_i64), _vp, _sz,
                                      _vp]
    L.m16_capacities.restype = ctypes.c_int
    L.m16_capacities.argtypes = [_vp, _i32, _i32, _i32, _f64, _f64, _vp, _vp, _vp, _vp]
    L.m16_fast_dice_workspace_bytes.restype = _sz
    L.m16_fast_dice_workspace_bytes.argtypes = [_i32]
    L.m16_fast_dice.restype = ctypes.c_int
    L.m16_fast_dice.argtypes = [ctypes.POINTER(_vp), _i32, _i64, _vp, ctypes.POINTER(_f64), _vp, _sz, _vp]
    L.m16_adjust_nonridge_signs_workspace_bytes.restype = _sz
    L.m16_adjust_nonridge_signs_workspace_bytes.argtypes = [_i32, _i32, _i32, _i64]
    L.m16_adjust_nonridge_signs_indexed.restype = ctypes.c_int
    L.m16_adjust_nonridge_signs_indexed.argtypes = [_vp, _i32, _i32, _i32, _vp, _vp, _i64, _vp, _vp, _sz, _vp]
    L.m16_batch_workspace_bytes.restype = _sz
    L.m16_batch_workspace_bytes.argtypes = [ctypes.POINTER(BatchVolume), _i32, ctypes.POINTER(BatchInstance), _i32]
    L.m16_batch_solve.restype = ctypes.c_int
    L.m16_batch_solve.argtypes = [ctypes.POINTER(BatchVolume), _i32, ctypes.POINTER(BatchInstance), _i32,
                                  ctypes.POINTER(CutParams), _vp, _vp, _vp, _sz, _vp, ctypes.POINTER(SolveStats)]
    L.m16_batch_begin.restype = ctypes.c_int
    L.m16_batch_begin.argtypes = [ctypes.POINTER(BatchVolume), _i32, ctypes.POINTER(BatchInstance), _i32,
                                  ctypes.POINTER(CutParams), _vp, _sz, _vp, ctypes.POINTER(_vp)]
    L.m16_batch_iterate.restype = ctypes.c_int
    L.m16_batch_iterate.argtypes = [_vp, _i32, _vp]
    L.m16_batch_end.restype = ctypes.c_int
    L.m16_batch_end.argtypes = [_vp, _vp, _vp, _vp]
    L.m16_server_request_bytes.restype = _sz
    L.m16_server_request_bytes.argtypes = [_i32, _i32, _i32, _i32]
    L.m16_server_table_bytes.restype = _sz
    L.m16_server_table_bytes.argtypes = [_i32, _i32]
    L.m16_server_create.restype = ctypes.c_int
    L.m16_server_create.argtypes = [ctypes.POINTER(CutParams), _i32, _i32, _vp, _sz, _vp, ctypes.POINTER(_vp)]
    L.m16_server_admit.restype = ctypes.c_int
    L.m16_server_admit.argtypes = [_vp, ctypes.POINTER(ServeRequest), ctypes.POINTER(_i32)]
    L.m16_server_step.restype = ctypes.c_int
    L.m16_server_step.argtypes = [_vp]
    L.m16_server_poll.restype = ctypes.c_int
    L.m16_server_poll.argtypes = [_vp, _vp, _vp, _vp, _i32, ctypes.POINTER(_i32)]
    L.m16_server_get_info.restype = ctypes.c_int
    L.m16_server_get_info.argtypes = [_vp, ctypes.POINTER(ServerInfo)]
    L.m16_server_destroy.restype = ctypes.c_int
    L.m16_server_destroy.argtypes = [_vp]
    L.m16_gvf_workspace_bytes.restype = _sz
    L.m16_gvf_workspace_bytes.argtypes = [_i32, _i32, _i32, _i32, _i32]
    L.m16_gvf_run.restype = ctypes.c_int
    L.m16_gvf_run.argtypes = [_vp, _vp, _i32, _i32, _i32, _vp, _f64, _f64, _i32, _i32, _i32, _f64, _i32, _vp,
                              ctypes.POINTER(_i32), ctypes.POINTER(_i32), _vp, _i32, ctypes.POINTER(_i32), _vp,
                              _sz, _vp]


def lib(build_if_missing: bool = True):
    """The loaded C-ABI library; builds it in-tree if it is absent."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.lib_path()
            if not os.path.exists(path):
                if not build_if_missing:
                    raise RuntimeError("CUDA library not built: %s" % path)
                path = _build.build()
            L = ctypes.CDLL(path)
            _declare(L)
            _lib = L
    return _lib


def status_string(status: int) -> str:
    return lib().m16_status_string(int(status)).decode()


def check(fn: str, status: int):
    if status != M16_OK:
        raise M16Error(fn, status)


# ---- torch glue ---------------------------------------------------------------

def torch_mod():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("miccai2016_gb300 needs a CUDA device (no CPU fallback)")
    return torch


def device():
    torch = torch_mod()
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr():
    torch = torch_mod()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t):
    """Device pointer of a torch tensor (or None)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def to_device_f32(a, shape=None):
    """numpy array / scalar / torch tensor -> contiguous float32 CUDA tensor."""
    torch = torch_mod()
    if isinstance(a, torch.Tensor):
        t = a.to(device=device(), dtype=torch.float32)
    else:
        arr = np.require(a, dtype=np.float32, requirements=["C", "A"])
        t = torch.from_numpy(arr).to(device())
    t = t.contiguous()
    if shape is not None and tuple(t.shape) != tuple(shape):
        t = t.reshape(shape)
    return t


def to_device_u8(a):
    torch = torch_mod()
    if isinstance(a, torch.Tensor):
        return a.to(device=device(), dtype=torch.uint8).contiguous()
    arr = np.require(a, dtype=np.uint8, requirements=["C", "A"])
    return torch.from_numpy(arr).to(device()).contiguous()


def workspace(nbytes: int):
    """A 256-byte-aligned device workspace (torch's caching allocator aligns
    to at least 512 bytes)."""
    torch = torch_mod()
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device())


def is_torch(a) -> bool:
    try:
        import torch
    except ImportError:  # pragma: no cover
        return False
    return isinstance(a, torch.Tensor)
