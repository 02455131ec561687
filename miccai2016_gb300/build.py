"""
Build recipe of the CUDA library: every csrc/*.cu translation unit is compiled
for sm_103a with nvcc (in parallel) and linked into
miccai2016_gb300/_lib/libmiccai2016_gb300.so, the C-ABI library declared in
include/miccai2016_gb300.h.  No cmake, one -gencode, static cudart.  The
host-only csrc/*.cpp files go through nvcc as plain C++ with multiply-add
contraction off (-ffp-contract=off): their floating-point sums must round
each product as numpy does, on x86 and Arm hosts alike.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
# M16_LIB_DIR builds/loads a tuning variant elsewhere; M16_NVCC_DEFINES adds
# -D flags (e.g. "-DM16_MF_ZB=4") to every translation unit of that variant.
OUT_DIR = os.environ.get("M16_LIB_DIR") or os.path.join(PKG_DIR, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
EXTRA_DEFINES = os.environ.get("M16_NVCC_DEFINES", "").split()
LIB_NAME = "libmiccai2016_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]
HOST_CPP_FLAGS = ["-O2", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off"]


def nvcc_path() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build the library")
    return cand


def lib_path() -> str:
    return os.path.join(OUT_DIR, LIB_NAME)


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(REPO_DIR, "include", "*.h"))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if stale) and return the path of the shared library."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu"))) + sorted(glob.glob(os.path.join(CSRC, "*.cpp")))
    if not srcs:
        raise RuntimeError("no CUDA sources under %s" % CSRC)
    out = lib_path()
    newest_hdr = max([os.path.getmtime(h) for h in _headers()] + [0.0])
    nvcc = nvcc_path()

    def compile_one(src):
        obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
        if (not force and os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
                and os.path.getmtime(obj) >= newest_hdr):
            return obj, False
        flags = HOST_CPP_FLAGS if src.endswith(".cpp") else ARCH + NVCC_FLAGS
        cmd = [nvcc] + flags + EXTRA_DEFINES + ["-c", src, "-o", obj]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, proc.stdout, proc.stderr))
        if verbose and proc.stderr.strip():
            print(proc.stderr)
        return obj, True

    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(compile_one, srcs))
    objs = [o for o, _ in results]
    rebuilt = any(r for _, r in results)
    if rebuilt or force or not os.path.exists(out) or any(os.path.getmtime(o) > os.path.getmtime(out) for o in objs):
        tmp = out + ".tmp"
        cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static"]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (proc.stdout, proc.stderr))
        os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(verbose=True))
