"""CPU checks of the pi program's host arithmetic (preclib_gb300/pi/bignum.cpp):
Newton reciprocal and exact division (with the reciprocal computed at the
minimum precision and above it), integer square root, and decimal conversion
(powers built inside or ahead of time), against Python integers.  The test program
tests/pi_host/bignum_check.cpp runs the same code on a schoolbook multiply,
built with 64-digit conversion leaves so that small numbers split over many
levels."""
import os
import random
import shutil
import subprocess
import sys

import pytest

if hasattr(sys, "set_int_max_str_digits"):
    sys.set_int_max_str_digits(0)  # decimal strings of numbers up to 30000 bits

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = [os.path.join(ROOT, "tests", "pi_host", "bignum_check.cpp"),
       os.path.join(ROOT, "preclib_gb300", "pi", "bignum.cpp")]


SANITIZE = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer", "-g"]


@pytest.fixture(scope="module", params=["plain", "sanitized"])
def run(request, tmp_path_factory):
    """The check program, plain and built with AddressSanitizer and
    UndefinedBehaviorSanitizer (any report fails the run: out-of-bounds or
    use-after-free on the limb buffers, leaks, signed overflow, shifts past
    the width)."""
    if not shutil.which("g++"):
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("bignum") / "bignum_check")
    flags = SANITIZE if request.param == "sanitized" else []
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-DPI_LEAF_DIGITS=64", *flags, "-o", exe] + SRC,
                       capture_output=True, text=True)
    if r.returncode and request.param == "sanitized":
        pytest.skip("no sanitizer runtime: " + r.stderr[-200:])
    assert r.returncode == 0, r.stderr
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="halt_on_error=1")

    def go(lines):
        r = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, timeout=600,
                           env=env)
        assert r.returncode == 0, r.stderr[-2000:]
        assert "runtime error" not in r.stderr and "Sanitizer" not in r.stderr, r.stderr[-2000:]
        return r.stdout.split("\n")[:len(lines)]
    return go


def h(x):
    return format(x, "x")


def _operands(rng):
    """(N, D) pairs: random sizes, D with all-ones and power-of-two shapes,
    N below D, N a multiple of D and one less than a multiple."""
    out = []
    for _ in range(60):
        nb = rng.randrange(1, 6000)
        db = rng.randrange(1, nb + 1)
        N = rng.getrandbits(nb) | (1 << (nb - 1))
        D = rng.getrandbits(db) | (1 << (db - 1))
        out.append((N, D))
    for db in (64, 65, 127, 128, 129, 1000, 3000):
        D = (1 << db) - 1
        out += [(rng.getrandbits(2 * db + 17) | 1, D), ((1 << (3 * db)) - 1, D), (1 << (2 * db), 1 << (db - 1))]
        q = rng.getrandbits(db + 5) | 1
        out += [(q * D, D), (q * D - 1, D), (D - 1, D), (D, D)]
    return out


def test_division(run):
    rng = random.Random(11)
    cases = _operands(rng)
    lines = ["divmod %s %s" % (h(N), h(D)) for N, D in cases]
    lines += ["divrecip %s %s %d" % (h(N), h(D), e) for (N, D), e in zip(cases, [0, 1, 64, 1000] * len(cases))]
    got = run(lines)
    for (N, D), g in zip(cases + cases, got):
        q, r = (int(x, 16) for x in g.split())
        assert (q, r) == divmod(N, D), (N.bit_length(), D.bit_length())


def test_isqrt(run):
    import math
    rng = random.Random(12)
    xs = [rng.getrandbits(rng.randrange(1, 9000)) | 1 for _ in range(60)]
    for b in (1, 2, 63, 64, 65, 128, 4000):
        s = rng.getrandbits(b) | (1 << (b - 1))
        xs += [s * s, s * s - 1, (s + 1) * (s + 1) - 1, 1 << (2 * b), (1 << (2 * b)) - 1]
    xs += [1, 2, 3, 4, 10005 * 10 ** 400]
    got = run(["isqrt %s" % h(x) for x in xs])
    for x, g in zip(xs, got):
        assert int(g, 16) == math.isqrt(x), x.bit_length()


def test_decimal(run):
    rng = random.Random(13)
    xs = [rng.getrandbits(rng.randrange(1, 20000)) for _ in range(40)]
    xs += [0, 1, 9, 10, 10 ** 64 - 1, 10 ** 64, 10 ** 128, 10 ** 1000 - 1, 10 ** 1000 + 1, 2 ** 8000]
    widths = [0, 1, 50, 3000]
    lines = ["dec %s %d" % (h(x), w) for x in xs for w in widths]
    got = run(lines)
    i = 0
    for x in xs:
        for w in widths:
            assert got[i] == str(x).zfill(w), (x.bit_length(), w)
            i += 1


def test_decimal_with_powers_ahead(run):
    """powers built for as many levels as needed, more, or fewer (then the
    conversion builds its own)"""
    rng = random.Random(14)
    xs = [rng.getrandbits(rng.randrange(100, 30000)) for _ in range(20)] + [3 * 10 ** 5000 + 7]
    lines, want = [], []
    for x in xs:
        need = len(str(x)) + 2
        levels = 0
        while (64 << levels) < need:
            levels += 1
        for L in (levels, levels + 2, max(0, levels - 2)):
            lines.append("decpre %s %d" % (h(x), L))
            want.append(str(x))
    assert run(lines) == want
