"""Builds the interposer (preclib_gb300/precn/prec_gpu_precn.cpp) over the
stand-in precn_t of this folder into a shared library for ctypes."""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIBDIR = os.path.join(ROOT, "preclib_gb300", "lib")

MUL_NTT_SYMBOL = "_Z7mul_nttRK7precn_tS1_"  # precn_t mul_ntt(const precn_t&, const precn_t&)
MUL_FFT_SYMBOL = "_Z7mul_fftRK7precn_tS1_"


def build(outdir: str) -> str:
    out = os.path.join(outdir, "libprecn_shim.so")
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-DCOUNT_FFTS=1", "-I" + HERE,
           "-I" + os.path.join(ROOT, "include"), os.path.join(ROOT, "preclib_gb300", "precn", "prec_gpu_precn.cpp"),
           os.path.join(HERE, "precn_shim.cpp"), "-L" + LIBDIR, "-lprecgpu", "-Wl,-rpath," + LIBDIR, "-o", out]
    subprocess.run(cmd, check=True)
    return out


def load(path: str) -> ctypes.CDLL:
    L = ctypes.CDLL(path)
    u64p = ctypes.POINTER(ctypes.c_uint64)
    L.shim_mul.argtypes = [ctypes.c_int, ctypes.c_int, u64p, ctypes.c_size_t, u64p, ctypes.c_size_t, u64p,
                           ctypes.POINTER(ctypes.c_int)]
    L.shim_mul.restype = ctypes.c_size_t
    L.shim_fft_counters.argtypes = [u64p, ctypes.POINTER(ctypes.c_double)]
    L.shim_fft_counters.restype = None
    return L
