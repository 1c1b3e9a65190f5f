"""CPU tests of the link-time wiring into preclib: the interposer that
defines mul_ntt / mul_fft on top of the C ABI builds, exports both symbols,
and with no device reaches the library (which refuses with its no-device
code) instead of any CPU multiply."""
import ctypes
import os
import subprocess
import sys

import pytest

from precn_shim import shim

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INTERPOSED = os.path.join(ROOT, "oracle", "_ref", "interposed")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="module")
def shim_path(tmp_path_factory):
    return shim.build(str(tmp_path_factory.mktemp("precn")))


def test_interposer_defines_both_multipliers(shim_path):
    L = ctypes.CDLL(shim_path)
    for sym in (shim.MUL_NTT_SYMBOL, shim.MUL_FFT_SYMBOL, "shim_mul", "shim_fft_counters"):
        assert hasattr(L, sym), sym


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device refusal")
def test_interposer_has_no_cpu_path(shim_path):
    """Without a device every product aborts with the library's error, like
    the reference's own failures (mul_ntt.cpp:135-136): nothing computes it
    on the CPU."""
    code = ("import sys, numpy as np; sys.path.insert(0, %r); from precn_shim import shim; "
            "L = shim.load(%r); a = np.arange(1, 301, dtype=np.uint64); out = np.zeros(600, np.uint64); "
            "import ctypes; z = ctypes.c_int(0); p = ctypes.POINTER(ctypes.c_uint64); "
            "L.shim_mul(1, 0, a.ctypes.data_as(p), 300, a.ctypes.data_as(p), 300, out.ctypes.data_as(p), "
            "ctypes.byref(z))") % (os.path.join(ROOT, "tests"), shim_path)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode != 0
    assert "prec_gpu: mul_fft: no usable CUDA device" in r.stderr


@pytest.mark.skipif(not os.path.exists(os.path.join(INTERPOSED, "fft_torture")),
                    reason="reference sources absent: interposed programs not built")
def test_reference_programs_link_to_the_gpu_path():
    """preclib's own fft_torture, test_opt_smoke and pi_chudnovsky, linked
    without src/mul_ntt.cpp and src/mul_fft.cpp: both symbols come from the
    interposer, and the library is what they call."""
    for prog in ("fft_torture", "test_opt_smoke", "pi_chudnovsky"):
        path = os.path.join(INTERPOSED, prog)
        syms = subprocess.run(["nm", path], capture_output=True, text=True, check=True).stdout
        assert " T " + shim.MUL_NTT_SYMBOL in syms, prog
        assert " T " + shim.MUL_FFT_SYMBOL in syms, prog
        assert " U prec_gpu_mul" in syms, prog
    if not _has_gpu():
        r = subprocess.run([os.path.join(INTERPOSED, "fft_torture")], capture_output=True, text=True,
                           timeout=120, cwd=INTERPOSED)
        assert r.returncode != 0
        assert "no usable CUDA device" in r.stderr
