"""CPU checks of the pi program: the golden table is complete and the
program refuses to run without a device (no CPU multiply behind it)."""
import json
import os
import subprocess

import pytest

from preclib_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(B.LIBDIR, B.PI_EXE)


def test_golden_table():
    runs = json.load(open(os.path.join(ROOT, "tests", "golden", "pi.json")))["runs"]
    assert [r["digits"] for r in runs] == [10 ** e for e in range(2, 9)]
    for r in runs:
        assert r["bytes"] == r["digits"] + 3  # "3." + digits + newline
        assert len(r["sha256"]) == 64


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device refusal")
def test_pi_program_needs_the_gpu():
    if not os.path.exists(EXE):
        pytest.skip("pi program not built")
    r = subprocess.run([EXE, "1000"], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0
    assert "no usable CUDA device" in r.stderr
