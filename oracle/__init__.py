"""Oracle package (test infrastructure only).

ctypes access to the C restatement of preclib's multiply (``liboracle.so``,
built from ``oracle_mul.c``) and, where the reference sources were present
when it was built, to the reference itself (``_ref/libprecref.so``).  Only
the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package.
"""
from .oracle import *  # noqa: F401,F403
