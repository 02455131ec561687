"""
Generates tests/golden/normalize.npz by running the reference's own
normalize (src/helpers/misc.py:63-114) on seeded inputs that reach every
branch: min-max, lower / upper / both percentiles, clipping on and off, the
dst_max-only and dst_min != 0 rescalings, a zero range, integer data.

The function's text is taken from the reference checkout and executed here
unchanged, with one alias the installed NumPy no longer has (np.float, a
name for the builtin float, i.e. float64).  It therefore runs with the
installed NumPy's promotion rules.  Needs the reference checkout:

    python tests/golden/make_normalize_golden.py [reference root]
"""
from __future__ import annotations

import ast
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MISC = os.path.join("src", "helpers", "misc.py")


def reference_normalize(ref_root):
    src = open(os.path.join(ref_root, MISC)).read()
    tree = ast.parse(src)
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "normalize")
    np_shim = types.ModuleType("np_shim")
    np_shim.__dict__.update({k: getattr(np, k) for k in dir(np) if not k.startswith("__")})
    np_shim.float = np.float64
    ns = {"np": np_shim}
    exec(compile(ast.Module(body=[fn], type_ignores=[]), MISC, "exec"), ns)
    return ns["normalize"]


def cases():
    rng = np.random.RandomState(20160101)
    f32 = rng.normal(0.3, 2.0, (7, 9, 11)).astype(np.float32)
    f64 = rng.uniform(-5, 5, (13, 17)).astype(np.float64)
    ints = rng.randint(-100, 400, (6, 5, 4)).astype(np.int32)
    const = np.full((4, 4, 4), 2.5, np.float32)
    frangi_like = np.abs(rng.standard_cauchy((8, 8, 8))).astype(np.float32) * 1e-3
    out = []
    for name, data in (("f32", f32), ("f64", f64), ("ints", ints), ("frangi_like", frangi_like)):
        out += [
            (name + "_minmax", data, dict()),
            (name + "_minmax_0_5", data, dict(dst_min=0.0, dst_max=5.0)),
            (name + "_minmax_m1_1", data, dict(dst_min=-1.0, dst_max=1.0)),
            (name + "_minmax_2_3_noclip", data, dict(dst_min=2.0, dst_max=3.0, clip=False)),
            (name + "_plow", data, dict(perc_low=5.0)),
            (name + "_pup", data, dict(perc_up=90.0)),
            (name + "_both", data, dict(perc_low=2.5, perc_up=97.5)),
            (name + "_both_noclip", data, dict(perc_low=10.0, perc_up=80.0, clip=False)),
            (name + "_both_m2_7", data, dict(dst_min=-2.0, dst_max=7.0, perc_low=1.0, perc_up=99.0)),
        ]
    out += [("const_minmax", const, dict()), ("const_shift", const, dict(dst_min=3.0, dst_max=4.0)),
            ("const_perc", const, dict(perc_low=10.0, perc_up=90.0))]
    return out


def main(argv):
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle.build import REF_ROOT
    ref_root = argv[1] if len(argv) > 1 else REF_ROOT
    norm = reference_normalize(ref_root)
    arrays = {}
    for name, data, kw in cases():
        arrays[name + "__in"] = data
        arrays[name + "__out"] = np.asarray(norm(data, **kw))
    path = os.path.join(HERE, "normalize.npz")
    np.savez_compressed(path, **arrays)
    print(path, len(arrays) // 2, "cases", os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(sys.argv)
