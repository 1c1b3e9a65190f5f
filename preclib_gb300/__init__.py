"""preclib_gb300 -- GB300-native large-operand multiply for preclib.

The product path is the sm_103a library ``lib/libprecgpu.so`` behind the C
ABI of ``include/prec_gpu.h``; this package is its Python host mirror
(ctypes binding, synthetic workload generators, build recipe).  There is
no CPU fallback anywhere in the package.
"""
from .native import (  # noqa: F401
    PrecGpuError,
    init,
    last_stats,
    mul,
    mul_device,
    ntt_log2,
    stream_check,
    strerror,
)

__all__ = ["PrecGpuError", "init", "last_stats", "mul", "mul_device", "ntt_log2",
           "stream_check", "strerror"]
