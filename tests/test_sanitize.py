"""The library's host C++ under AddressSanitizer and UndefinedBehaviorSanitizer
(CPU, no device).

The host-side translation units (context and plans, batch form, serving
loop, tuner, no-allocation entry point) are compiled again with
-fsanitize=address,undefined and linked with the kernel objects of the
normal build; then the CPU tests of the C ABI and of the tuning table run
against that library, with the sanitizer runtime preloaded into the Python
process.  Any report (out-of-bounds access, use after free, overflow of a
signed value, a shift past the width) fails the run.  The paths covered are
those that need no device: argument and size refusals, plan selection for
every transform length, the tuning table's validation and its text format
(save, load, malformed files), error strings.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from preclib_gb300 import build as B  # noqa: E402

HOST_TUS = ("prec_gpu_host.cu", "prec_gpu_batch.cu", "prec_gpu_serve.cu", "prec_gpu_tune.cu", "prec_gpu_noalloc.cu")
SAN = ["-fsanitize=address", "-fsanitize=undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer"]
# nvcc splits -Xcompiler arguments at commas: one flag per -Xcompiler
XSAN = [x for f in SAN for x in ("-Xcompiler", f)]


def _runtime(name):
    p = subprocess.run(["gcc", "-print-file-name=" + name], capture_output=True, text=True).stdout.strip()
    return p if os.path.isabs(p) and os.path.exists(p) else None


def test_host_code_under_sanitizers(tmp_path):
    try:
        nvcc = B.nvcc()
    except RuntimeError:
        pytest.skip("no nvcc")
    asan, ubsan = _runtime("libasan.so"), _runtime("libubsan.so")
    if not (asan and ubsan and shutil.which("gcc")):
        pytest.skip("no sanitizer runtime")
    kernel_objs = [os.path.join(B.OBJDIR, os.path.basename(s) + ".o") for s in B.sources()
                   if os.path.basename(s) not in HOST_TUS]
    if not all(os.path.exists(o) for o in kernel_objs):
        pytest.skip("the library is not built (run build() first)")

    def compile_host(name):
        out = str(tmp_path / (name + ".o"))
        cmd = [nvcc, *B.ARCH, *B.NVCC_FLAGS, *XSAN, "-I", os.path.join(ROOT, "include"),
               "-c", os.path.join(B.CSRC, name), "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        return out

    with ThreadPoolExecutor(len(HOST_TUS)) as ex:
        host_objs = list(ex.map(compile_host, HOST_TUS))
    lib = str(tmp_path / "libprecgpu_san.so")
    r = subprocess.run([nvcc, *B.ARCH, "-shared", "-o", lib, *host_objs, *kernel_objs, "-lcudart", *XSAN], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]

    runner = ("import sys; sys.path.insert(0, %r); from preclib_gb300 import native; native.LIB_PATH = %r; "
              "assert native.lib()._name == native.LIB_PATH; "
              "import pytest; sys.exit(pytest.main(['-q', '-p', 'no:cacheprovider', '-m', 'not gpu', %r, %r]))"
              % (ROOT, lib, os.path.join(ROOT, "tests", "test_abi.py"), os.path.join(ROOT, "tests", "test_tune.py")))
    env = dict(os.environ, LD_PRELOAD=asan + ":" + ubsan,
               # the interpreter itself is not instrumented: its allocations
               # are not ours to report as leaks
               ASAN_OPTIONS="detect_leaks=0:protect_shadow_gap=0", UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1",
               CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-c", runner], capture_output=True, text=True, env=env, timeout=600)
    out = r.stdout + r.stderr
    assert r.returncode == 0, out[-3000:]
    assert "runtime error" not in out and "ERROR: AddressSanitizer" not in out, out[-3000:]
    assert " passed" in out
