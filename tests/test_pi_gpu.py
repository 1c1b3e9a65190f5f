"""GPU parity of the pi program (preclib_gb300/pi): its output file is
byte-identical to preclib's own pi program at 10^2 .. 10^8 digits (hashes
generated from the reference by tests/golden/make_pi_golden.py; 10^8 is
the workload size of the Chudnovsky benchmark, a 100,000,003-byte file)."""
import hashlib
import json
import os
import subprocess

import pytest

from preclib_gb300 import build as B

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(B.LIBDIR, B.PI_EXE)


def _runs():
    with open(os.path.join(ROOT, "tests", "golden", "pi.json")) as f:
        return {r["digits"]: r for r in json.load(f)["runs"]}


@pytest.mark.parametrize("digits", [100, 1000, 10000, 100000, 1000000, 10000000, 100000000])
def test_pi_digits_match_reference(gpu, tmp_path, digits):
    want = _runs()[digits]
    out = tmp_path / "pi.txt"
    r = subprocess.run([EXE, str(digits), "--phases", "--file", str(out)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    data = out.read_bytes()
    assert len(data) == want["bytes"]
    assert hashlib.sha256(data).hexdigest() == want["sha256"]
    assert data.startswith(b"3.14159265")


def test_pi_digits_host_newton(gpu, tmp_path):
    """The host-resident Newton steps (every product staged through host
    memory), kept for comparison, give the same digits."""
    want = _runs()[1000000]
    out = tmp_path / "pi.txt"
    env = dict(os.environ, PI_GB300_HOST_NEWTON="1")
    r = subprocess.run([EXE, "1000000", "--file", str(out)], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr
    data = out.read_bytes()
    assert hashlib.sha256(data).hexdigest() == want["sha256"]


def test_pi_device_forms_match_host_forms(gpu):
    """pi_gb300 --self-check: the device-resident decimal conversion, square
    root and exact division agree with the host-resident forms of
    bignum.cpp on zero, powers of ten at the conversion's leaf and level
    sizes and their neighbours, runs of nines and zeros, all-ones limbs,
    perfect squares and their neighbours, quotients at the correction's edges
    and random numbers."""
    r = subprocess.run([EXE, "--self-check"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "0 disagreements" in r.stderr, r.stderr
