"""
Generates the golden fixtures in tests/golden/*.npz by running the reference's
own OpenCL C kernels (compiled for the CPU through oracle/ref_shim; needs the
reference checkout) on the seeded inputs of tests/golden/inputs.py.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from oracle import oracle as O  # noqa: E402
import inputs as I  # noqa: E402


def make_maxflow():
    for name in I.MAXFLOW_CASES:
        inp, kw = I.maxflow_case(name)
        u, iters, resid = O.ref_maxflow_solve(inp["img"], inp["quats"], inp["eigs"], inp["alpha"], inp["cs"],
                                              inp["ct"], labels=inp["labels"], scaling=inp["scaling"], **kw)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, u=u, iterations=np.int64(iters), residuals=np.asarray(resid, np.float64))
        print(name, u.shape, iters, len(resid), os.path.getsize(path))


def make_gvf():
    for name in I.GVF_CASES:
        v, kw = I.gvf_case(name)
        g, iters, mags = O.ref_gvf_run(v, **kw)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, g=g, iterations=np.int64(iters), mags=np.asarray(mags, np.float64))
        print(name, g.shape, iters, len(mags), os.path.getsize(path))


def make_frangi():
    for name in I.FRANGI_CASES:
        img, kw = I.frangi_case(name)
        val, quat, c = O.ref_frangi(img, **kw)
        sig = O.frangi_scales(kw["scales"], np.ones(3) if kw["voxel_size"] is None else kw["voxel_size"])
        h = np.stack([O.hessian(img, s) for s in sig[:1]])
        e = np.empty_like(h)
        for k in range(len(h)):
            ek = h[k].reshape(-1, 6).copy()
            O.ref().ref_eigs(O.ctypes.c_long(ek.shape[0]), O._ptr(ek), O._ptr(ek))
            e[k] = ek.reshape(h[k].shape)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, val=val, quat=quat, c=c, hessian=h, eigs=e)
        print(name, val.shape, c, os.path.getsize(path))


def make_directions():
    d = I.directions_case()
    out = {}
    for th in (0.01, 0.3):
        out["ridge_%g" % th] = O.ref_detect_ridges(d["resp"], d["quats"], th)
    out["main"] = O.ref_extract_main_directions(d["quats"])
    out["complete"] = O.ref_complete_transformations(d["vecs"])
    out["adjust_iso"] = O.ref_adjust_nonridge_signs(d["vecs"], d["coords"], d["rdirs"], (1, 1, 1))
    out["adjust_aniso"] = O.ref_adjust_nonridge_signs(d["vecs"], d["coords"], d["rdirs"], (1.5, 0.7, 1.2))
    path = os.path.join(HERE, "directions.npz")
    np.savez_compressed(path, **out)
    print("directions", os.path.getsize(path))


if __name__ == "__main__":
    if O.ref() is None:
        raise SystemExit("the reference checkout is needed to generate fixtures")
    which = sys.argv[1:] or ["maxflow", "gvf", "frangi", "directions"]
    if "maxflow" in which:
        make_maxflow()
    if "gvf" in which:
        make_gvf()
    if "frangi" in which:
        make_frangi()
    if "directions" in which:
        make_directions()
