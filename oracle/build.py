"""
oracle/build.py -- build recipe for the CPU checker (TEST INFRASTRUCTURE ONLY).

* build_oracle(): compiles the C restatement in oracle/*.c into
  oracle/_build/liboracle.so (gcc, OpenMP, no fused multiply-add).
* build_ref(): when the reference checkout is present, compiles the
  reference's own OpenCL C kernels with g++ through oracle/ref_shim into
  oracle/_ref/libref.so.  The .cl text is read in place and piped into the
  compiler; the few OpenCL-only constructs g++ cannot parse (vector literals,
  one vector-condition ternary, two assigned `const int2`) are rewritten in
  memory first.  No reference source is written anywhere.

Both libraries are loaded by oracle/oracle.py.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
# the reference checkout: $MICCAI2016_REFERENCE, else a "reference" directory
# beside this repository's root
REF_ROOT = os.environ.get("MICCAI2016_REFERENCE") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))
ORACLE_SOURCES = ["maxflow.c", "gvf.c", "frangi.c", "directions.c"]

CFLAGS = ["-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-std=gnu11", "-Wall",
          "-Wno-unused-function", "-Wno-unknown-pragmas"]


def _run(cmd, stdin_text=None):
    proc = subprocess.run(cmd, input=stdin_text, text=True, capture_output=True)
    if proc.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), proc.stdout, proc.stderr))
    return proc


def oracle_lib_path() -> str:
    return os.path.join(BUILD_DIR, "liboracle.so")


def ref_lib_path() -> str:
    return os.path.join(REF_DIR, "libref.so")


def build_oracle(force: bool = False) -> str:
    """Compile the C restatement into oracle/_build/liboracle.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    out = oracle_lib_path()
    srcs = [os.path.join(HERE, s) for s in ORACLE_SOURCES if os.path.exists(os.path.join(HERE, s))]
    deps = srcs + [os.path.join(HERE, "qmath.h")]
    if not force and os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        _run(["gcc"] + CFLAGS + ["-c", src, "-o", obj])
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = out + ".tmp"
    _run(["gcc", "-shared", "-fopenmp", "-o", tmp] + objs + ["-lm"])
    os.replace(tmp, out)
    return out


# --- the reference, compiled through the shim --------------------------------

_SHIM_GLOBALS = (
    "static double shim_RCC, shim_RS0, shim_RS1, shim_RS2, shim_SS0, shim_SS1, shim_SS2,"
    " shim_SQ0, shim_SQ1, shim_SQ2, shim_MU, shim_DT, shim_RSS0, shim_RSS1, shim_RSS2,"
    " shim_THRESHOLD;\n"
)
_MF_MACROS = ["RCC=(shim_RCC)", "RS0=(shim_RS0)", "RS1=(shim_RS1)", "RS2=(shim_RS2)",
              "SS0=(shim_SS0)", "SS1=(shim_SS1)", "SS2=(shim_SS2)", "SQEVAL0=(shim_SQ0)",
              "SQEVAL1=(shim_SQ1)", "SQEVAL2=(shim_SQ2)"]
_GVF_MACROS = ["MU=(shim_MU)", "DT=(shim_DT)", "RSS0=(shim_RSS0)", "RSS1=(shim_RSS1)",
               "RSS2=(shim_RSS2)"]

# (namespace, reference file, kind macro, suffix, extra -D)
_REF_UNITS = [
    ("mf_c_u", "src/clcode-anisotropic/update_qp.cl", "REF_KIND_UPDATE_QP", "_c_u", _MF_MACROS + ["CONST_EVALS"]),
    ("mf_c_s", "src/clcode-anisotropic/update_qp.cl", "REF_KIND_UPDATE_QP", "_c_s",
     _MF_MACROS + ["CONST_EVALS", "SUPERVISED"]),
    ("mf_p_u", "src/clcode-anisotropic/update_qp.cl", "REF_KIND_UPDATE_QP", "_p_u", _MF_MACROS),
    ("mf_p_s", "src/clcode-anisotropic/update_qp.cl", "REF_KIND_UPDATE_QP", "_p_s", _MF_MACROS + ["SUPERVISED"]),
    ("gvf", "src/clcode/gvf.cl", "REF_KIND_GVF", "", _GVF_MACROS),
    ("conv", "src/clcode/convolve_naive.cl", "REF_KIND_CONVOLVE", "", []),
    # qfrangi_gpu.py:300-302: ascending absolute value, 50 sweeps
    ("eig", "src/clcode/qeigs.cl", "REF_KIND_EIGS", "",
     ["eigcmp(current,extreme)=(fabs(current) < fabs(extreme))", "MAXITER=50"]),
    ("frangi", "src/clcode/frangi.cl", "REF_KIND_FRANGI", "", []),
    ("ridges", "src/clcode/detect_ridges.cl", "REF_KIND_RIDGES", "", ["THRESHOLD=(shim_THRESHOLD)"]),
    ("adjust", "src/clcode/adjust_directions.cl", "REF_KIND_ADJUST", "", ["THRESHOLD=(-1)"]),
]


def _rewrite_opencl(text: str, name: str) -> str:
    """In-memory rewrites of the OpenCL-only syntax that C++ cannot parse."""
    text = re.sub(r"\((float3|int3|uint3|float4|int2)\)\s*\(", r"make_\1(", text)
    if name == "ridges":
        old = "crnRel_k == 1 ? pos_j : 1 - pos_j"
        assert text.count(old) == 1, "unexpected detect_ridges.cl layout"
        text = text.replace(old, "shim_vselect(crnRel_k == 1, pos_j, 1 - pos_j)")
    if name == "adjust":
        assert text.count("const int2 i2d;") == 2, "unexpected adjust_directions.cl layout"
        text = text.replace("const int2 i2d;", "int2 i2d;")
    return text


def reference_available() -> bool:
    return os.path.isdir(os.path.join(REF_ROOT, "src", "clcode"))


def build_ref(force: bool = False) -> str | None:
    """Compile the reference kernels into oracle/_ref/libref.so (None if absent)."""
    if not reference_available():
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    out = ref_lib_path()
    shim_deps = [os.path.join(HERE, "ref_shim", f) for f in ("clshim.hpp", "launch.inc")] + [__file__]
    if not force and os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in shim_deps):
        return out
    inc = os.path.join(REF_ROOT, "src", "clcode")

    def compile_unit(unit):
        ns, rel, kind, suffix, defs = unit
        with open(os.path.join(REF_ROOT, rel), "r") as f:
            cl_text = f.read()
        cl_text = _rewrite_opencl(cl_text, ns)
        tu = ('#include "clshim.hpp"\n' + _SHIM_GLOBALS + "namespace %s {\n" % ns + cl_text +
              "\n}\n" + '#include "launch.inc"\n')
        obj = os.path.join(REF_DIR, ns + ".o")
        cmd = ["g++", "-x", "c++", "-", "-std=gnu++17", "-O2", "-fopenmp", "-ffp-contract=off",
               "-fPIC", "-w", "-Wno-narrowing", "-I", os.path.join(HERE, "ref_shim"), "-I", inc,
               "-D", kind, "-D", "REF_NS=%s" % ns, "-D", "REF_SUFFIX=%s" % suffix,
               "-c", "-o", obj]
        for d in defs:
            cmd += ["-D", d]
        _run(cmd, stdin_text=tu)
        return obj

    with ThreadPoolExecutor(max_workers=8) as ex:
        objs = list(ex.map(compile_unit, _REF_UNITS))
    tmp = out + ".tmp"
    _run(["g++", "-shared", "-fopenmp", "-o", tmp] + objs)
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
