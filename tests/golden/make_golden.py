"""Generates tests/golden/products.json from the reference itself.

Runs preclib's own mul_ntt / mul_fft / operator* (compiled from its sources
by oracle/build_ref.sh into oracle/_ref/libprecref.so) on the operand
generators of the reference's tests and of the benchmark configurations, and
records per product: the SHA-256 of the an+bn output limbs (little-endian
bytes), the normalised length, a few head/tail limbs and, for mul_fft, the
reference's max rounding distance.  Run from the repository root:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import numpy as np  # noqa: E402

import oracle as O  # noqa: E402
import patterns  # noqa: E402


def digest(out: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(out, dtype="<u8").tobytes()).hexdigest()


def record(name, gen, fn):
    a, b = patterns.make(gen)
    if fn == "sqr":
        out, err = O.ref_sqr(a), None
    elif fn == "fft":
        out, err = O.ref_mul_fft(a, b)
    elif fn == "ntt":
        out, err = O.ref_mul_ntt(a, b), None
    else:
        out, err = O.ref_mul(a, b), None
    nz = np.flatnonzero(out)
    rec = {"name": name, "gen": gen, "ref_fn": fn, "limbs": int(len(out)),
           "rsiz": int(nz[-1] + 1) if len(nz) else 0, "sha256": digest(out),
           "head": [int(x) for x in out[:4]], "tail": [int(x) for x in out[-4:]]}
    if err is not None:
        rec["fft_max_err"] = err
    return rec


def main():
    if O.ref_lib() is None:
        sys.exit("oracle/_ref/libprecref.so missing: run oracle/build_ref.sh first")
    recs = []
    # benchmark configurations (SplitMix64, top limb nonzero)
    recs.append(record("cfg1_8192x8192_ntt", dict(kind="splitmix64", seed_a=1, seed_b=2, an=8192, bn=8192), "ntt"))
    recs.append(record("cfg2_1Mx1M_ntt", dict(kind="splitmix64", seed_a=3, seed_b=4, an=1 << 20, bn=1 << 20), "ntt"))
    recs.append(record("cfg2_3000x3000_fft", dict(kind="splitmix64", seed_a=5, seed_b=6, an=3000, bn=3000), "fft"))
    # above 1M x 1M: the 64-bit-digit plan over the second five-prime set
    # (2^23 points), the largest requests of the serving configuration
    recs.append(record("big_4Mx4M_ntt", dict(kind="splitmix64", seed_a=25, seed_b=26, an=1 << 22, bn=1 << 22), "ntt"))
    # test/bench_ntt.cpp sizes (1024..65536 limbs, seeds 1000+n, 2000+n)
    n = 1024
    while n <= 65536:
        recs.append(record("bench_ntt_%d" % n, dict(kind="lcg64", seed_a=1000 + n, seed_b=2000 + n, an=n, bn=n), "ntt"))
        n <<= 1
    # test/test_prec.cpp cross-algorithm matrix (445-478)
    for i, base in enumerate((32, 128, 512, 2048)):
        for seedoff, bn in ((3000, base), (3100, base + base // 4), (3150, base + base // 3),
                            (3200, base + base // 2), (3300, base * 2), (3400, base * 3)):
            seed = seedoff + i
            gen = dict(kind="lcg32", seed_a=seed, seed_b=seed + 1009, an=base, bn=bn)
            recs.append(record("test_prec_%d_%d" % (base, bn), gen, "mul"))
    # test/test_opt_smoke.cpp:48-50 (2049 x 2039 via mul_fft)
    recs.append(record("opt_smoke_fft_2049x2039", dict(kind="lcg64", seed_a=750, seed_b=760, an=2049, bn=2039), "fft"))
    # test/fft_torture.cpp: every shape x pattern, both multipliers
    for (an, bn) in patterns.TORTURE_SHAPES:
        for p in patterns.TORTURE_PATTERNS:
            gen = dict(kind="torture", pattern=p[0], an=an, bn=bn)
            recs.append(record("torture_%s_%dx%d_fft" % (p[0], an, bn), gen, "fft"))
            recs.append(record("torture_%s_%dx%d_ntt" % (p[0], an, bn), gen, "ntt"))
    # NTT band edges and unbalanced shapes
    for (an, bn, s) in ((6145, 6145, 40), (6145, 12290, 41), (12289, 7000, 42), (20000, 10001, 43),
                        (100000, 77777, 44), (262144, 262144, 45), (300000, 150001, 46)):
        recs.append(record("edge_%dx%d_ntt" % (an, bn), dict(kind="splitmix64", seed_a=s, seed_b=s + 100, an=an, bn=bn), "ntt"))
    # precn_sqr (src/mul_basic.cpp:193-204): mul_fft(a, a) above 192 limbs at
    # every size, Karatsuba below; the operand is `a` of the generator
    for (an, s) in ((100, 60), (193, 61), (3000, 62), (6144, 63), (6145, 64), (8192, 65), (20000, 66),
                    (65536, 67), (1 << 18, 68)):
        recs.append(record("sqr_%d" % an, dict(kind="splitmix64", seed_a=s, seed_b=s, an=an, bn=an), "sqr"))
    for an in (6144, 20000):
        recs.append(record("sqr_ones_%d" % an, dict(kind="torture", pattern="all-ones", an=an, bn=an), "sqr"))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "products.json")
    with open(path, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "reference": "preclib src/*.cpp (g++ -O3, COUNT_FFTS=1)",
                   "products": recs}, f, indent=1)
    print("wrote %d records to %s" % (len(recs), path))


if __name__ == "__main__":
    main()
