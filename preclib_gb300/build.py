"""Build recipe of the native library (nvcc, sm_103a only, in-tree output).

``python -m preclib_gb300.build`` compiles every translation unit under
``csrc/`` in parallel with one ``-gencode`` and links ``lib/libprecgpu.so``.
The output is git-ignored; it is rebuilt on each machine (x86 here, Arm on
the GPU hosts).
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(PKG, "_build")
LIBNAME = "libprecgpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-Xcudafe", "--diag_suppress=177"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build preclib_gb300")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _compile(src: str, extra) -> str:
    obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-I", os.path.join(PKG, "..", "include"),
           "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj


def build(verbose: bool = False, extra=()) -> str:
    """Compile and link lib/libprecgpu.so; returns its path."""
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    out = os.path.join(LIBDIR, LIBNAME)
    tmp = out + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, out)
    build_pi()
    if verbose:
        print("built", out)
    return out


PI_SOURCES = ("bignum.cpp", "pi_chudnovsky.cpp", "pi_kernels.cu", "dnat.cu", "ddec.cu")
PI_EXE = "pi_gb300"


def build_pi(extra=()) -> str:
    """The pi program (pi/*.cpp, host C++) linked against lib/libprecgpu.so."""
    srcs = [os.path.join(PKG, "pi", f) for f in PI_SOURCES]
    out = os.path.join(LIBDIR, PI_EXE)
    cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-pthread", *extra,
           "-I", os.path.join(PKG, "..", "include"), *srcs, "-L", LIBDIR, "-lprecgpu",
           "-Xlinker", "-rpath=" + LIBDIR, "-o", out + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("pi program build failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
