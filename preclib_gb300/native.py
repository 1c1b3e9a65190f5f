"""ctypes binding of ``lib/libprecgpu.so`` (the C ABI of include/prec_gpu.h).

There is no fallback: importing the binding without the built library, or
calling it without a CUDA device, raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

LIB_PATH = os.path.join(_build.LIBDIR, _build.LIBNAME)

OK = 0
E_ARG, E_TOO_LARGE, E_NOMEM, E_CUDA, E_TIMEOUT, E_FFT_ROUNDING, E_NODEV, E_INTERNAL = range(1, 9)

# Every symbol include/prec_gpu.h declares (checked by the CPU tests).
EXPORTS = (
    "prec_gpu_init", "prec_gpu_shutdown", "prec_gpu_mul", "prec_gpu_mul_ntt",
    "prec_gpu_mul_device", "prec_gpu_stream_check", "prec_gpu_last_stats",
    "prec_gpu_ntt_log2", "prec_gpu_strerror", "prec_gpu_mul_device_profile",
    "prec_gpu_stage_name", "prec_gpu_mul_device_noalloc", "prec_gpu_mul_fft",
    "prec_gpu_fft_digit_bits", "prec_gpu_batch_create", "prec_gpu_batch_run", "prec_gpu_batch_info",
    "prec_gpu_batch_destroy", "prec_gpu_mul_batch", "prec_gpu_serve_create", "prec_gpu_serve_submit",
    "prec_gpu_serve_wait", "prec_gpu_serve_drain", "prec_gpu_serve_stats", "prec_gpu_serve_destroy",
    "prec_gpu_sqr", "prec_gpu_autotune", "prec_gpu_tune_get", "prec_gpu_tune_set", "prec_gpu_tune_reset",
    "prec_gpu_tune_save", "prec_gpu_tune_load", "prec_gpu_launch_count", "prec_gpu_set_wide_digits",
    "prec_gpu_set_block_limbs",
)

_u64p = ctypes.POINTER(ctypes.c_uint64)


class Stats(ctypes.Structure):
    _fields_ = [("path", ctypes.c_int), ("log2_n", ctypes.c_int), ("primes", ctypes.c_int),
                ("digit_bits", ctypes.c_int), ("limbs_a", ctypes.c_size_t), ("limbs_b", ctypes.c_size_t),
                ("fft_max_distance", ctypes.c_double), ("device_ms", ctypes.c_double)]


class Product(ctypes.Structure):
    """prec_gpu_product_t: device pointers and limb counts of one product."""
    _fields_ = [("a", ctypes.c_void_p), ("an", ctypes.c_size_t), ("b", ctypes.c_void_p),
                ("bn", ctypes.c_size_t), ("out", ctypes.c_void_p)]


class TuneEntry(ctypes.Structure):
    """prec_gpu_tune_entry_t: kernel configuration of one NTT length."""
    _fields_ = [("log2_n", ctypes.c_int), ("log2_cols", ctypes.c_int), ("col_group", ctypes.c_int),
                ("col_radix_cap", ctypes.c_int), ("row_radix_cap", ctypes.c_int), ("rows_per_cta", ctypes.c_int),
                ("split_primes", ctypes.c_int),
                ("ms", ctypes.c_float), ("default_ms", ctypes.c_float)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServeStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double),
                ("max_ms", ctypes.c_double), ("products_per_s", ctypes.c_double),
                ("peak_bytes", ctypes.c_size_t), ("peak_in_flight", ctypes.c_int)]


class PrecGpuError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        super().__init__("%s: %s (code %d)" % (what or "prec_gpu", strerror(code), code))


_LIB = None


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("preclib_gb300 native library missing at %s; run "
                              "`python -m preclib_gb300.build` (no CPU fallback exists)" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        L.prec_gpu_init.argtypes = [ctypes.c_int]
        L.prec_gpu_init.restype = ctypes.c_int
        L.prec_gpu_shutdown.argtypes = []
        L.prec_gpu_shutdown.restype = None
        for name in ("prec_gpu_mul", "prec_gpu_mul_ntt", "prec_gpu_mul_fft"):
            f = getattr(L, name)
            f.argtypes = [_u64p, ctypes.c_size_t, _u64p, ctypes.c_size_t, _u64p]
            f.restype = ctypes.c_int
        L.prec_gpu_sqr.argtypes = [_u64p, ctypes.c_size_t, _u64p]
        L.prec_gpu_sqr.restype = ctypes.c_int
        L.prec_gpu_launch_count.argtypes = []
        L.prec_gpu_launch_count.restype = ctypes.c_uint64
        L.prec_gpu_set_wide_digits.argtypes = [ctypes.c_int]
        L.prec_gpu_set_wide_digits.restype = ctypes.c_int
        L.prec_gpu_set_block_limbs.argtypes = [ctypes.c_size_t]
        L.prec_gpu_set_block_limbs.restype = ctypes.c_size_t
        L.prec_gpu_autotune.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(TuneEntry), ctypes.c_size_t,
                                        ctypes.POINTER(ctypes.c_size_t)]
        L.prec_gpu_autotune.restype = ctypes.c_int
        L.prec_gpu_tune_get.argtypes = [ctypes.c_int, ctypes.POINTER(TuneEntry)]
        L.prec_gpu_tune_get.restype = ctypes.c_int
        L.prec_gpu_tune_set.argtypes = [ctypes.POINTER(TuneEntry)]
        L.prec_gpu_tune_set.restype = ctypes.c_int
        L.prec_gpu_tune_reset.argtypes = []
        L.prec_gpu_tune_reset.restype = ctypes.c_int
        L.prec_gpu_tune_save.argtypes = [ctypes.c_char_p]
        L.prec_gpu_tune_save.restype = ctypes.c_int
        L.prec_gpu_tune_load.argtypes = [ctypes.c_char_p]
        L.prec_gpu_tune_load.restype = ctypes.c_int
        L.prec_gpu_mul_device.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                          ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
        L.prec_gpu_mul_device.restype = ctypes.c_int
        L.prec_gpu_stream_check.argtypes = [ctypes.c_void_p]
        L.prec_gpu_stream_check.restype = ctypes.c_int
        L.prec_gpu_last_stats.argtypes = [ctypes.POINTER(Stats)]
        L.prec_gpu_last_stats.restype = ctypes.c_int
        L.prec_gpu_fft_digit_bits.argtypes = [ctypes.c_size_t, ctypes.c_size_t]
        L.prec_gpu_fft_digit_bits.restype = ctypes.c_int
        L.prec_gpu_ntt_log2.argtypes = [ctypes.c_size_t, ctypes.c_size_t]
        L.prec_gpu_ntt_log2.restype = ctypes.c_int
        L.prec_gpu_mul_device_profile.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                                  ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.POINTER(ctypes.c_float),
                                                  ctypes.POINTER(ctypes.c_int)]
        L.prec_gpu_mul_device_profile.restype = ctypes.c_int
        L.prec_gpu_mul_device_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                                  ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
        L.prec_gpu_mul_device_noalloc.restype = ctypes.c_int
        L.prec_gpu_batch_create.argtypes = [ctypes.POINTER(Product), ctypes.c_size_t,
                                            ctypes.POINTER(ctypes.c_void_p)]
        L.prec_gpu_batch_create.restype = ctypes.c_int
        L.prec_gpu_batch_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.prec_gpu_batch_run.restype = ctypes.c_int
        L.prec_gpu_batch_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t),
                                          ctypes.POINTER(ctypes.c_size_t)]
        L.prec_gpu_batch_info.restype = ctypes.c_int
        L.prec_gpu_batch_destroy.argtypes = [ctypes.c_void_p]
        L.prec_gpu_batch_destroy.restype = None
        L.prec_gpu_mul_batch.argtypes = [ctypes.POINTER(Product), ctypes.c_size_t, ctypes.c_void_p]
        L.prec_gpu_mul_batch.restype = ctypes.c_int
        L.prec_gpu_serve_create.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        L.prec_gpu_serve_create.restype = ctypes.c_int
        L.prec_gpu_serve_submit.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                            ctypes.c_size_t, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
        L.prec_gpu_serve_submit.restype = ctypes.c_int
        L.prec_gpu_serve_wait.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double,
                                          ctypes.POINTER(ctypes.c_double)]
        L.prec_gpu_serve_wait.restype = ctypes.c_int
        L.prec_gpu_serve_drain.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.prec_gpu_serve_drain.restype = ctypes.c_int
        L.prec_gpu_serve_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ServeStats)]
        L.prec_gpu_serve_stats.restype = ctypes.c_int
        L.prec_gpu_serve_destroy.argtypes = [ctypes.c_void_p]
        L.prec_gpu_serve_destroy.restype = None
        L.prec_gpu_stage_name.argtypes = [ctypes.c_int, ctypes.c_int]
        L.prec_gpu_stage_name.restype = ctypes.c_char_p
        L.prec_gpu_strerror.argtypes = [ctypes.c_int]
        L.prec_gpu_strerror.restype = ctypes.c_char_p
        _LIB = L
    return _LIB


def strerror(code: int) -> str:
    try:
        return lib().prec_gpu_strerror(code).decode()
    except ImportError:
        return "error %d" % code


def check(code: int, what: str = "") -> None:
    if code != OK:
        raise PrecGpuError(code, what)


def _arr(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint64)


def _p(a: np.ndarray):
    return a.ctypes.data_as(_u64p)


def init(device: int = -1) -> None:
    check(lib().prec_gpu_init(device), "prec_gpu_init")


def mul(a, b, ntt: bool = False, fft: bool = False) -> np.ndarray:
    """Product of two host limb vectors (an+bn limbs), computed on the GPU:
    band routing by default, or the NTT / FP64 FFT band forced."""
    a, b = _arr(a), _arr(b)
    out = np.empty(max(len(a) + len(b), 1), dtype=np.uint64)
    f = lib().prec_gpu_mul_ntt if ntt else (lib().prec_gpu_mul_fft if fft else lib().prec_gpu_mul)
    check(f(_p(a), len(a), _p(b), len(b), _p(out)), "prec_gpu_mul")
    return out[: len(a) + len(b)]


def sqr(a) -> np.ndarray:
    """Square of a host limb vector (2*len(a) limbs), computed on the GPU."""
    a = _arr(a)
    out = np.empty(max(2 * len(a), 1), dtype=np.uint64)
    check(lib().prec_gpu_sqr(_p(a), len(a), _p(out)), "prec_gpu_sqr")
    return out[: 2 * len(a)]


def autotune(kmin: int = 13, kmax: int = 26):
    """Tunes the kernel configuration of NTT lengths 2^kmin .. 2^kmax on the
    current device; returns one dict per length (chosen config and times)."""
    cap = 32
    arr = (TuneEntry * cap)()
    n = ctypes.c_size_t(0)
    check(lib().prec_gpu_autotune(kmin, kmax, arr, cap, ctypes.byref(n)), "prec_gpu_autotune")
    return [arr[i].as_dict() for i in range(min(n.value, cap))]


def launch_count() -> int:
    """Kernel launches the library has issued in this process."""
    return int(lib().prec_gpu_launch_count())


def set_block_limbs(limbs: int) -> int:
    """Block size (limbs) above which a product runs blocked (0: the default,
    2^24); returns the previous setting."""
    return int(lib().prec_gpu_set_block_limbs(limbs))


def set_wide_digits(on: bool) -> bool:
    """64-bit digits over five primes for single NTT-band products (True, the
    default) or 32-bit digits over three primes; returns the previous setting."""
    return bool(lib().prec_gpu_set_wide_digits(1 if on else 0))


def tune_get(log2_n: int) -> dict:
    e = TuneEntry()
    check(lib().prec_gpu_tune_get(log2_n, ctypes.byref(e)), "prec_gpu_tune_get")
    return e.as_dict()


def tune_set(**cfg) -> None:
    """Installs a configuration: keys of TuneEntry (log2_n required)."""
    e = TuneEntry(**{k: v for k, v in cfg.items() if k in dict(TuneEntry._fields_)})
    check(lib().prec_gpu_tune_set(ctypes.byref(e)), "prec_gpu_tune_set")


def tune_reset() -> None:
    check(lib().prec_gpu_tune_reset(), "prec_gpu_tune_reset")


def tune_save(path: str) -> None:
    check(lib().prec_gpu_tune_save(path.encode()), "prec_gpu_tune_save")


def tune_load(path: str) -> None:
    check(lib().prec_gpu_tune_load(path.encode()), "prec_gpu_tune_load")


def mul_device(a_ptr: int, an: int, b_ptr: int, bn: int, out_ptr: int, stream: int = 0) -> None:
    """Enqueue a product on device pointers (e.g. torch tensors' data_ptr())."""
    check(lib().prec_gpu_mul_device(a_ptr, an, b_ptr, bn, out_ptr, stream or None),
          "prec_gpu_mul_device")


def mul_device_profile(a_ptr: int, an: int, b_ptr: int, bn: int, out_ptr: int, stream: int = 0):
    """Run one product on device pointers; returns [(kernel name, ms), ...]."""
    ms = (ctypes.c_float * 8)()
    n = ctypes.c_int(0)
    check(lib().prec_gpu_mul_device_profile(a_ptr, an, b_ptr, bn, out_ptr, stream or None, ms,
                                            ctypes.byref(n)), "prec_gpu_mul_device_profile")
    path = 0 if n.value == 1 else 1
    return [(lib().prec_gpu_stage_name(path, i).decode(), float(ms[i])) for i in range(n.value)]


def stream_check(stream: int = 0) -> None:
    check(lib().prec_gpu_stream_check(stream or None), "prec_gpu_stream_check")


def last_stats() -> Stats:
    s = Stats()
    check(lib().prec_gpu_last_stats(ctypes.byref(s)))
    return s


def fft_digit_bits(an: int, bn: int) -> int:
    return lib().prec_gpu_fft_digit_bits(an, bn)


def ntt_log2(an: int, bn: int) -> int:
    return lib().prec_gpu_ntt_log2(an, bn)


class Batch:
    """A planned batch of device-resident products (prec_gpu_batch_t).

    items: sequence of (a_ptr, an, b_ptr, bn, out_ptr) device pointers."""

    def __init__(self, items):
        arr = (Product * max(len(items), 1))(*[Product(*it) for it in items])
        self._h = ctypes.c_void_p()
        check(lib().prec_gpu_batch_create(arr, len(items), ctypes.byref(self._h)), "prec_gpu_batch_create")

    def run(self, stream: int = 0) -> None:
        check(lib().prec_gpu_batch_run(self._h, stream or None), "prec_gpu_batch_run")

    def info(self):
        c, b = ctypes.c_size_t(), ctypes.c_size_t()
        check(lib().prec_gpu_batch_info(self._h, ctypes.byref(c), ctypes.byref(b)))
        return c.value, b.value

    def close(self) -> None:
        if self._h:
            lib().prec_gpu_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mul_batch(items, stream: int = 0) -> None:
    """One-shot batch (synchronous) of (a_ptr, an, b_ptr, bn, out_ptr) products."""
    arr = (Product * max(len(items), 1))(*[Product(*it) for it in items])
    check(lib().prec_gpu_mul_batch(arr, len(items), stream or None), "prec_gpu_mul_batch")


class Server:
    """Serving loop (prec_gpu_server_t): device-resident requests admitted by
    HBM footprint into `slots` concurrent streams."""

    def __init__(self, hbm_budget_bytes: int, slots: int = 8):
        self._h = ctypes.c_void_p()
        check(lib().prec_gpu_serve_create(hbm_budget_bytes, slots, ctypes.byref(self._h)), "prec_gpu_serve_create")

    def submit(self, a_ptr: int, an: int, b_ptr: int, bn: int, out_ptr: int) -> int:
        t = ctypes.c_uint64()
        check(lib().prec_gpu_serve_submit(self._h, a_ptr, an, b_ptr, bn, out_ptr, ctypes.byref(t)),
              "prec_gpu_serve_submit")
        return t.value

    def wait(self, ticket: int, timeout_s: float = 60.0) -> float:
        ms = ctypes.c_double()
        check(lib().prec_gpu_serve_wait(self._h, ticket, timeout_s, ctypes.byref(ms)), "prec_gpu_serve_wait")
        return ms.value

    def drain(self, timeout_s: float = 300.0) -> None:
        check(lib().prec_gpu_serve_drain(self._h, timeout_s), "prec_gpu_serve_drain")

    def stats(self) -> ServeStats:
        st = ServeStats()
        check(lib().prec_gpu_serve_stats(self._h, ctypes.byref(st)))
        return st

    def close(self) -> None:
        if self._h:
            lib().prec_gpu_serve_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
