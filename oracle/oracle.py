"""
oracle/oracle.py -- numpy front end of the CPU checker.

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
baseline legs of bench.py import this module; the product package never does.

Two libraries sit behind it:
* liboracle.so -- the C restatement in oracle/*.c (the "port"), built
  everywhere, including on machines without the reference checkout;
* libref.so    -- the reference's own OpenCL C kernels compiled through
  oracle/ref_shim (only where the reference checkout exists).  It is used to
  pin the port and to generate the committed golden fixtures.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_u16p = np.ctypeslib.ndpointer(dtype=np.uint16, flags="C_CONTIGUOUS")
_i64 = ctypes.c_int64
_vp = ctypes.c_void_p

_lib = None
_ref = None


def lib():
    """The C restatement (liboracle.so), built on first use."""
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        _lib = ctypes.CDLL(path)
        _declare_oracle(_lib)
    return _lib


def ref():
    """The reference kernels through the shim (libref.so), or None."""
    global _ref
    if _ref is None:
        path = _build.ref_lib_path()
        if not os.path.exists(path):
            path = _build.build_ref()
        if path is None or not os.path.exists(path):
            return None
        _ref = ctypes.CDLL(path)
    return _ref


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_vp)


def _f32(a):
    return np.require(a, dtype=np.float32, requirements=["C", "A"])


def _declare_oracle(L):
    L.oracle_maxflow_solve.restype = ctypes.c_int
    L.oracle_maxflow_solve.argtypes = [_vp] * 8 + [_i64, _i64, _i64, _vp, ctypes.c_double,
                                                   ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                                   ctypes.c_double, _vp, _vp, _vp]
    L.oracle_sum_abs.restype = ctypes.c_double
    L.oracle_sum_abs.argtypes = [_vp, _i64]
    L.oracle_mf_update_p.restype = None
    L.oracle_mf_update_p.argtypes = [_i64, _i64, _i64, _vp, ctypes.c_double, ctypes.c_double, _vp] + [_vp] * 7
    L.oracle_mf_update_u.restype = None
    L.oracle_mf_update_u.argtypes = [_i64, _i64, _i64, _vp, ctypes.c_double, ctypes.c_double] + [_vp] * 9
    L.oracle_mf_update_tmp.restype = None
    L.oracle_mf_update_tmp.argtypes = [_i64, _vp, ctypes.c_double, _vp, _vp]
    L.oracle_convolve.restype = None
    L.oracle_convolve.argtypes = [ctypes.c_int, _i64, _i64, _i64, _vp, _vp, _vp, ctypes.c_int]
    L.oracle_hessian.restype = None
    L.oracle_hessian.argtypes = [_i64, _i64, _i64, _vp, _vp, _vp, _vp]
    L.oracle_eigs.restype = None
    L.oracle_eigs.argtypes = [_i64, _vp, _vp]
    L.oracle_max_norm.restype = ctypes.c_float
    L.oracle_max_norm.argtypes = [_i64, _vp]
    L.oracle_update_vesselness.restype = None
    L.oracle_update_vesselness.argtypes = [_i64, _vp, _vp, _vp, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                           ctypes.c_int]
    L.oracle_frangi.restype = None
    L.oracle_frangi.argtypes = [_i64, _i64, _i64, _vp, ctypes.c_int, _vp, _vp, ctypes.c_float, ctypes.c_float,
                                ctypes.c_float, ctypes.c_int, _vp, _vp, _vp]
    L.oracle_detect_ridges.restype = None
    L.oracle_detect_ridges.argtypes = [_i64, _i64, _i64, ctypes.c_double, _vp, _vp, _vp]
    L.oracle_extract_main_directions.restype = None
    L.oracle_extract_main_directions.argtypes = [_i64, _vp, _vp]
    L.oracle_complete_transformations.restype = None
    L.oracle_complete_transformations.argtypes = [_i64, _vp, _vp]
    L.oracle_adjust_nonridge_signs.restype = None
    L.oracle_adjust_nonridge_signs.argtypes = [_i64, _i64, _i64, _vp, _vp, _vp, _i64, _vp]
    L.oracle_prim_mst.restype = None
    L.oracle_prim_mst.argtypes = [_vp, _i64, _vp, _vp]
    L.oracle_gvf_time_step.restype = ctypes.c_double
    L.oracle_gvf_time_step.argtypes = [_vp, ctypes.c_double, ctypes.c_int]
    L.oracle_gvf_run.restype = ctypes.c_int
    L.oracle_gvf_run.argtypes = [_vp, _vp, _i64, _i64, _i64, _vp, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_double, ctypes.c_int, _vp, _vp, _vp]


# ----------------------------------------------------------------------------
# max-flow
# ----------------------------------------------------------------------------

def mf_consts(scaling=(1, 1, 1), cc=0.2, steps=0.11, sqevals=(1.0, 1.0, 1.0)):
    """RCC, RS0-2, SS0-2, SQEVAL0-2 as the reference derives them
    (src/processing/continuous_cut_anisotropic_gpu.py:104-129)."""
    scaling = np.asarray(scaling, dtype=np.float64)
    rs = 1.0 / scaling
    smin = np.min(scaling)
    ss = steps / scaling * smin ** 2
    rcc = 1.0 / (cc * smin ** 2)
    return np.array([rcc, rs[0], rs[1], rs[2], ss[0], ss[1], ss[2],
                     sqevals[0], sqevals[1], sqevals[2]], dtype=np.float64)


def _split_eigs(eigs, shape):
    """sqrt of a constant 3-tuple or of a per-voxel (z,y,x,3) array, as
    continuous_cut_anisotropic_gpu.py:216-221 and 246-251 arrange them."""
    sq = np.sqrt(np.asanyarray(eigs))
    if sq.ndim == 1:
        return np.ascontiguousarray(sq, dtype=np.float64), None
    return None, _f32(sq.reshape(-1, 3))


def maxflow_solve(img, quats, eigs, alpha, cs, ct, labels=None, scaling=None, cc=0.2, steps=0.11,
                  num_iter=1000, update=1, error_bound=1e-4):
    """One CmfCutQAnisotropicGpu.execute() solve on the CPU.

    Returns (u, iterations, residuals) where residuals lists every checked
    value of cc * mean|div(hp) - p_s + p_t|."""
    img = _f32(img)
    shape = img.shape
    n = img.size
    sqc, sqp = _split_eigs(eigs, shape)
    if not isinstance(alpha, np.ndarray):
        alpha = np.multiply(alpha, np.ones(shape), dtype=np.float32)
    alpha = _f32(alpha)
    cs, ct = _f32(cs), _f32(ct)
    q = _f32(quats).reshape(-1, 3)
    lab = None if labels is None else np.require(labels, dtype=np.uint8, requirements=["C", "A"])
    sc = np.asarray((1, 1, 1) if scaling is None else scaling, dtype=np.float64)
    u = np.empty(shape, np.float32)
    n_checks = ctypes.c_int(0)
    max_checks = (num_iter // max(update, 1)) + 2
    resid = np.zeros(max_checks, np.float64)
    iters = lib().oracle_maxflow_solve(_ptr(img), _ptr(q), None if sqc is None else _ptr(sqc), _ptr(sqp),
                                       _ptr(alpha), _ptr(cs), _ptr(ct), _ptr(lab), shape[0], shape[1],
                                       shape[2], _ptr(sc), cc, steps, num_iter, update, error_bound,
                                       _ptr(u), _ptr(resid), ctypes.byref(n_checks))
    return u, int(iters), resid[:n_checks.value].copy()


def sum_abs(x):
    x = _f32(x).ravel()
    return float(lib().oracle_sum_abs(_ptr(x), x.size))


def mf_update_p(hp, tmp, quats, eigs, alpha, scaling=(1, 1, 1), cc=0.2, steps=0.11):
    """In-place update_p on hp = [hp0, hp1, hp2] (each (z,y,x) float32)."""
    shape = tmp.shape
    sqc, sqp = _split_eigs(eigs, shape)
    sc = np.asarray(scaling, dtype=np.float64)
    lib().oracle_mf_update_p(shape[0], shape[1], shape[2], _ptr(sc), cc, steps,
                             None if sqc is None else _ptr(sqc), _ptr(hp[0]), _ptr(hp[1]), _ptr(hp[2]),
                             _ptr(_f32(tmp)), _ptr(_f32(quats)), _ptr(sqp), _ptr(_f32(alpha)))


def mf_update_u(hp, tmp, cs, ct, pt, u, labels=None, scaling=(1, 1, 1), cc=0.2, steps=0.11):
    shape = tmp.shape
    sc = np.asarray(scaling, dtype=np.float64)
    lab = None if labels is None else np.require(labels, dtype=np.uint8, requirements=["C", "A"])
    lib().oracle_mf_update_u(shape[0], shape[1], shape[2], _ptr(sc), cc, steps, _ptr(hp[0]), _ptr(hp[1]),
                             _ptr(hp[2]), _ptr(tmp), _ptr(_f32(cs)), _ptr(_f32(ct)), _ptr(pt), _ptr(u),
                             _ptr(lab))


def mf_update_tmp(tmp, u, scaling=(1, 1, 1), cc=0.2):
    sc = np.asarray(scaling, dtype=np.float64)
    lib().oracle_mf_update_tmp(tmp.size, _ptr(sc), cc, _ptr(tmp), _ptr(_f32(u)))


# --- the same, through the reference kernels ----------------------------------

def ref_mf_kernels(const_evals: bool, supervised: bool):
    """(update_p, update_u, update_tmp) of the shim-compiled update_qp.cl."""
    R = ref()
    if R is None:
        return None
    suf = ("_c" if const_evals else "_p") + ("_s" if supervised else "_u")
    return (getattr(R, "ref_update_p" + suf), getattr(R, "ref_update_u" + suf),
            getattr(R, "ref_update_tmp" + suf))


def ref_maxflow_solve(img, quats, eigs, alpha, cs, ct, labels=None, scaling=None, cc=0.2, steps=0.11,
                      num_iter=1000, update=1, error_bound=1e-4):
    """The reference's solve loop (continuous_cut_anisotropic_gpu.py:198-344)
    driving the reference's own kernels; the residual uses the port's
    sum_abs.  Returns (u, iterations, residuals)."""
    img = _f32(img)
    shape = img.shape
    n = img.size
    sq = np.sqrt(np.asanyarray(eigs))
    const = sq.ndim == 1
    kp, ku, kt = ref_mf_kernels(const, labels is not None)
    sc = (1, 1, 1) if scaling is None else scaling
    k = mf_consts(sc, cc, steps, sq if const else (1.0, 1.0, 1.0))
    if not isinstance(alpha, np.ndarray):
        alpha = np.multiply(alpha, np.ones(shape), dtype=np.float32)
    alpha, cs, ct = _f32(alpha), _f32(cs), _f32(ct)
    if const:
        e = _f32(quats)
    else:
        e = np.empty(shape + (6,), np.float32)
        e[..., :3] = sq
        e[..., 3:] = quats
    lab = None if labels is None else np.require(labels, dtype=np.uint8, requirements=["C", "A"])
    hp = [np.zeros(shape, np.float32) for _ in range(3)]
    pt = np.fmin(cs, ct)
    u = np.require(np.divide(img, np.max(img) + np.finfo(img.dtype).tiny), dtype=np.float32,
                   requirements=["C", "A"])
    tmp = np.zeros(shape, np.float32)
    d0, d1, d2 = shape
    kt(ctypes.c_long(n), _ptr(k), _ptr(tmp), _ptr(u))
    resid = []
    it = 0
    for it in range(num_iter):
        kp(d0, d1, d2, _ptr(k), _ptr(hp[0]), _ptr(hp[1]), _ptr(hp[2]), _ptr(tmp), _ptr(e), _ptr(alpha))
        ku(d0, d1, d2, _ptr(k), _ptr(hp[0]), _ptr(hp[1]), _ptr(hp[2]), _ptr(tmp), _ptr(cs), _ptr(ct),
           _ptr(pt), _ptr(u), _ptr(lab))
        if update > 0 and not it % update:
            err = sum_abs(tmp) / (n * k[0])
            resid.append(err)
            if np.isnan(err) or err < error_bound:
                return u, it + 1, np.array(resid)
        kt(ctypes.c_long(n), _ptr(k), _ptr(tmp), _ptr(u))
    return u, num_iter, np.array(resid)


# ----------------------------------------------------------------------------
# gradient vector flow
# ----------------------------------------------------------------------------

def gvf_time_step(voxel_size, mu):
    vs = np.asarray(np.multiply(voxel_size, np.ones(3)), dtype=np.float64)
    return float(lib().oracle_gvf_time_step(_ptr(vs), mu, 3))


def gvf_run(vfield, mu, maxiter, update, tol=0.0, normalize=False, voxel_size=None, response=None):
    """GvfGpu(vfield, params, voxel_size, response).execute() on the CPU.
    Returns (gvf (z,y,x,3) float32, iterations, mean-|delta| log)."""
    v = _f32(vfield)
    assert v.ndim == 4 and v.shape[-1] == 3
    shape = v.shape[:3]
    vs = np.asarray(np.ones(3) if voxel_size is None else np.multiply(voxel_size, np.ones(3)), np.float64)
    r = None if response is None else _f32(response)
    g = np.empty_like(v)
    mags = np.zeros(maxiter // max(update, 1) + 2, np.float64)
    nm = ctypes.c_int(0)
    it = lib().oracle_gvf_run(_ptr(v), _ptr(r), shape[0], shape[1], shape[2], _ptr(vs), mu, maxiter, update,
                              tol, int(bool(normalize)), _ptr(g), _ptr(mags), ctypes.byref(nm))
    return g, int(it), mags[:nm.value].copy()


def ref_gvf_run(vfield, mu, maxiter, update, tol=0.0, normalize=False, voxel_size=None, response=None):
    """The reference's GVF loop (gradient_vector_flow.py:179-232) driving the
    reference's own gvf.cl kernels through the shim."""
    R = ref()
    v = _f32(vfield)
    shape = v.shape[:3]
    n = int(np.prod(shape))
    vs = np.asarray(np.ones(3) if voxel_size is None else np.multiply(voxel_size, np.ones(3)), np.float64)
    dt = np.minimum(0.99, (np.min(vs) ** 3) / (2.01 ** 3 * mu))
    rss = 1. / (vs ** 2)
    k = np.array([mu, dt, rss[0], rss[1], rss[2]], np.float64)
    vc = [np.ascontiguousarray(v[..., c]) for c in range(3)]
    r = np.empty(shape, np.float32)
    if response is None:
        R.ref_gvf_response(ctypes.c_long(n), _ptr(r), _ptr(vc[0]), _ptr(vc[1]), _ptr(vc[2]))
    else:
        r[...] = response
    g = [np.zeros(shape, np.float32) for _ in range(3)]
    e = [np.zeros(shape, np.float32) for _ in range(3)]
    mags = []
    it = 0
    for it in range(int(maxiter)):
        R.ref_gvf_delta(shape[0], shape[1], shape[2], _ptr(k), _ptr(e[0]), _ptr(e[1]), _ptr(e[2]), _ptr(g[0]),
                        _ptr(g[1]), _ptr(g[2]), _ptr(vc[0]), _ptr(vc[1]), _ptr(vc[2]), _ptr(r))
        R.ref_gvf_update(ctypes.c_long(n), _ptr(k), _ptr(g[0]), _ptr(g[1]), _ptr(g[2]), _ptr(e[0]), _ptr(e[1]),
                         _ptr(e[2]))
        if not it % update:
            m = np.empty(shape, np.float32)
            R.ref_gvf_mag_delta(ctypes.c_long(n), _ptr(m), _ptr(e[0]), _ptr(e[1]), _ptr(e[2]))
            mag = sum_abs(m) / n
            mags.append(mag)
            if mag < tol:
                it += 1
                break
    else:
        it = int(maxiter)
    if normalize:
        R.ref_gvf_normalize(ctypes.c_long(n), _ptr(g[0]), _ptr(g[1]), _ptr(g[2]))
    return np.stack(g, axis=-1), it, np.array(mags)


# ----------------------------------------------------------------------------
# Frangi vesselness
# ----------------------------------------------------------------------------

def gauss_taps(sigma, order, scaling_factor=1.0, n_sigmas=4, round_up=False):
    """GaussianFilter3D._gauss_kernel_with (qfrangi_gpu.py:158-185), float32."""
    sigma_sq = sigma ** 2

    def gaussian(x):
        result = np.exp(-.5 * x ** 2 / sigma_sq)
        return result / np.sum(result)

    orders = [lambda x: gaussian(x),
              lambda x: gaussian(x) * (-x) / (sigma_sq),
              lambda x: gaussian(x) * (x ** 2 - sigma_sq) / (sigma_sq ** 2),
              lambda x: gaussian(x) * x * (3 * sigma_sq - x ** 2) / (sigma_sq ** 3)]
    x_max = int(np.ceil(n_sigmas * sigma)) if round_up else int(n_sigmas * sigma + 0.5)
    x_s = np.arange(-x_max, x_max + 1)
    return np.require(scaling_factor * orders[order](x_s), np.float32, ["C", "A"])


def frangi_scales(scales, voxel_size):
    """M x 3 per-axis sigmas in voxels (qfrangi_gpu.py:590-592)."""
    scales_mm = np.linspace(*scales).reshape(-1, 1)
    scaling = np.divide(1., voxel_size).reshape(1, -1)
    return np.dot(scales_mm, scaling)


def scale_taps(sigma3, gamma=1.0):
    """taps[axis][order] (order 0..2; index 3 unused) and radii of one scale,
    with the scale-space factor sigma ** (order * gamma) (qfrangi_gpu.py:136-142)."""
    taps = []
    radius = []
    for a in range(3):
        s = float(sigma3[a])
        row = [gauss_taps(s, o, s ** (o * gamma)) for o in range(3)]
        row.append(row[0])
        taps.append(row)
        radius.append(len(row[0]) // 2)
    return taps, radius


def _tap_ptr_array(taps_list):
    arrs = [t for scale in taps_list for axis in scale for t in axis]
    ptrs = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
    return ptrs, arrs


def convolve(volume, axis, taps):
    v = _f32(volume)
    out = np.empty_like(v)
    t = _f32(taps)
    lib().oracle_convolve(axis, v.shape[0], v.shape[1], v.shape[2], _ptr(out), _ptr(v), _ptr(t), len(t) // 2)
    return out


def hessian(img, sigma3):
    """N x 6 Hessian (00, 11, 22, 01, 02, 12) of one scale."""
    img = _f32(img)
    taps, radius = scale_taps(sigma3)
    ptrs, keep = _tap_ptr_array([taps])
    rad = np.asarray(radius, np.int32)
    h = np.empty(img.shape + (6,), np.float32)
    lib().oracle_hessian(img.shape[0], img.shape[1], img.shape[2], _ptr(img), ptrs, _ptr(rad), _ptr(h))
    return h


def eigs(h6):
    """Jacobi eigendecomposition: [l1, l2, l3 (ascending |l|), squeezed quaternion]."""
    h = _f32(h6)
    out = np.empty_like(h)
    lib().oracle_eigs(h.size // 6, _ptr(h), _ptr(out))
    return out


def frangi(img, scales, voxel_size=None, alpha=0.5, beta=0.5, c=None, bright=True):
    """VesselnessCalculation/FeatureFilter on the CPU: (vesselness, squeezed
    quaternions, c per scale).  `scales` is the (start, stop, number) triple
    in mm of VesselnessCalculation.Parameters."""
    img = _f32(img)
    vs = np.ones(3) if voxel_size is None else np.multiply(voxel_size, np.ones(3))
    sig = frangi_scales(scales, vs)
    per = [scale_taps(s) for s in sig]
    ptrs, keep = _tap_ptr_array([p[0] for p in per])
    rad = np.asarray([p[1] for p in per], np.int32).ravel()
    val = np.empty(img.shape, np.float32)
    quat = np.empty(img.shape + (3,), np.float32)
    cu = np.zeros(len(sig), np.float32)
    lib().oracle_frangi(img.shape[0], img.shape[1], img.shape[2], _ptr(img), len(sig), ptrs, _ptr(rad), alpha,
                        beta, -1.0 if c is None else float(c), int(bool(bright)), _ptr(val), _ptr(quat), _ptr(cu))
    return val, quat, cu


def ref_frangi(img, scales, voxel_size=None, alpha=0.5, beta=0.5, c=None, bright=True):
    """The reference's scale loop (qfrangi_gpu.py:511-580, 208-271, 383-439)
    over its own convolve_naive.cl, qeigs.cl and frangi.cl kernels."""
    R = ref()
    img = _f32(img)
    shape = img.shape
    n = img.size
    d0, d1, d2 = shape
    vs = np.ones(3) if voxel_size is None else np.multiply(voxel_size, np.ones(3))
    val = np.full(shape, -np.inf, np.float32)
    quat = np.zeros(shape + (3,), np.float32)
    cus = []
    for s in frangi_scales(scales, vs):
        taps, radius = scale_taps(s)
        h = np.empty((6, n), np.float32)
        for i in range(3):
            for j in range(i + 1):
                order = [0, 0, 0]
                order[i] = 1
                order[j] += 1
                a = img.copy()
                b = np.empty_like(a)
                for ax in range(3):
                    t = taps[ax][order[ax]]
                    R.ref_convolve(ax, d0, d1, d2, _ptr(b), _ptr(a), _ptr(t), radius[ax])
                    a, b = b, a
                h[i if i == j else 2 + i + j] = a.ravel()
        e = np.require(h.T, np.float32, ["C", "A"])
        R.ref_eigs(ctypes.c_long(n), _ptr(e), _ptr(e))
        if c is None:
            nrm = np.empty(n, np.float32)
            R.ref_calculate_norm(ctypes.c_long(n), _ptr(nrm), _ptr(e))
            cc = np.float32(0.5 * np.fmax.reduce(nrm))
        else:
            cc = np.float32(c)
        cus.append(cc)
        R.ref_update_vesselness(ctypes.c_long(n), _ptr(val), _ptr(quat), _ptr(e), ctypes.c_float(0.5 if alpha is None else alpha),
                                ctypes.c_float(beta), ctypes.c_float(cc), int(bool(bright)))
    return val, quat, np.array(cus, np.float32)


# ----------------------------------------------------------------------------
# direction kernels
# ----------------------------------------------------------------------------

def detect_ridges(resp, quat3, threshold):
    resp = _f32(resp)
    q = _f32(quat3)
    out = np.empty_like(resp)
    lib().oracle_detect_ridges(resp.shape[0], resp.shape[1], resp.shape[2], float(threshold), _ptr(out),
                               _ptr(resp), _ptr(q))
    return out


def extract_main_directions(quat3):
    q = _f32(quat3)
    out = np.empty_like(q)
    lib().oracle_extract_main_directions(q.size // 3, _ptr(out), _ptr(q))
    return out


def complete_transformations(dirs3):
    d = _f32(dirs3)
    out = np.empty_like(d)
    lib().oracle_complete_transformations(d.size // 3, _ptr(out), _ptr(d))
    return out


def adjust_nonridge_signs(dirs3, coords, rdirs, scaling=(1, 1, 1)):
    d = _f32(dirs3).copy()
    c = np.require(coords, np.uint16, ["C", "A"])
    r = _f32(rdirs)
    sc = np.asarray(np.multiply(scaling, np.ones(3)), np.float32)
    lib().oracle_adjust_nonridge_signs(d.shape[0], d.shape[1], d.shape[2], _ptr(d), _ptr(c), _ptr(r), len(c),
                                       _ptr(sc))
    return d


def _image_8192(values, dtype):
    """to_cl_image_8192 (cl_helpers.py:46-81) as the flat [row][8192][4] list."""
    n = len(values)
    rows = ((n - 1) >> 13) + 1
    out = np.zeros((rows * 8192, 4), dtype)
    out[:n, :3] = values
    return out


def ref_detect_ridges(resp, quat3, threshold):
    resp = _f32(resp)
    out = np.empty_like(resp)
    ref().ref_detect_ridges(resp.shape[0], resp.shape[1], resp.shape[2], ctypes.c_double(threshold), _ptr(out),
                            _ptr(resp), _ptr(_f32(quat3)))
    return out


def ref_extract_main_directions(quat3):
    q = _f32(quat3).copy()
    ref().ref_extract_main_directions(ctypes.c_long(q.size // 3), _ptr(q), _ptr(q))
    return q


def ref_complete_transformations(dirs3):
    d = _f32(dirs3).copy()
    ref().ref_complete_transformations(ctypes.c_long(d.size // 3), _ptr(d), _ptr(d))
    return d


def ref_adjust_nonridge_signs(dirs3, coords, rdirs, scaling=(1, 1, 1)):
    d = _f32(dirs3).copy()
    ci = _image_8192(np.asarray(coords), np.uint16)
    di = _image_8192(np.asarray(rdirs), np.float32)
    sc = np.asarray(np.multiply(scaling, np.ones(3)), np.float32)
    ref().ref_adjust_nonridge_signs(d.shape[0], d.shape[1], d.shape[2], _ptr(d), _ptr(ci), _ptr(di), _ptr(sc),
                                    len(coords))
    return d


def prim_mst_edges(points_scaled):
    """oracle_prim_mst: the (lo, hi) edges of the stable minimum spanning tree
    of float64 points (n x 3, already scaled by the voxel size)."""
    pts = np.require(points_scaled, dtype=np.float64, requirements=["C", "A"])
    n = len(pts)
    lo = np.zeros(max(n - 1, 0), np.int64)
    hi = np.zeros(max(n - 1, 0), np.int64)
    lib().oracle_prim_mst(_ptr(pts), n, _ptr(lo), _ptr(hi))
    return lo, hi
