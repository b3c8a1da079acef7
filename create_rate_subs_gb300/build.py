"""Build libcrs.so (the sm_103a kernels + C ABI) in-tree with nvcc.

    python -m create_rate_subs_gb300.build [--force]

Each .cu file in csrc/ is compiled in parallel for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), each .cpp file (host-only
code) by the host C++ compiler, then everything is linked into
create_rate_subs_gb300/lib/libcrs.so with the CUDA runtime linked
statically, so that loading it needs nothing beyond the driver.
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libcrs.so")
BUILD = os.path.join(HERE, "_build")
REPO = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
          "--expt-relaxed-constexpr", "-I", os.path.join(REPO, "include")]
# Per-file extra flags.  The strict FP64 kernels and the thermo utilities
# must not contract a*b+c into FMA: they reproduce the reference's operation
# order.
EXTRA = {"crs_fp64_strict.cu": ["-fmad=false"],
         # thermo utilities in the emitted operand order, bit for bit
         "crs_dydt.cu": ["-fmad=false"]}
# Host-only sources: the reentrant per-state functions, which must round
# every operation as the reference's emitted C does (no contraction into
# FMA, no fast math), whatever the host architecture's default.
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
              "-I", os.path.join(REPO, "include")]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    p = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(p):
        return p
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def cxx():
    for name in ("g++", "c++"):
        p = shutil.which(name)
        if p:
            return p
    raise RuntimeError("no host C++ compiler (g++) found")


def _stale(force):
    if force or not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for d in (CSRC, os.path.join(REPO, "include")):
        for f in os.listdir(d):
            if os.path.getmtime(os.path.join(d, f)) > t:
                return True
    return os.path.getmtime(__file__) > t


def build(force=False, verbose=False):
    """Compile and link libcrs.so if any source is newer; return its path."""
    if not _stale(force):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        if src.endswith(".cpp"):
            cmd = [cxx()] + HOST_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        else:
            cmd = ([cc] + ARCH + COMMON + EXTRA.get(src, [])
                   + ["-c", os.path.join(CSRC, src), "-o", obj])
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, res.stdout, res.stderr))
        if verbose and (res.stdout or res.stderr):
            print(res.stdout + res.stderr)
        return obj

    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n" + res.stdout + res.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
