"""Generates tests/golden/pi.json: SHA-256 and length of the output file of
preclib's own pi program (pi/pi_chudnovsky.cpp, compiled from its sources
by `oracle/build_ref.sh pi` into oracle/_ref/pi_ref) at 10^2 .. 10^7
digits (`pi_ref D --file F`; the 10^7 run takes about 1.5 minutes).  The
10^8-digit entry is the recorded result of the same program at 10^8
digits (about 37 minutes on one x86 core); pass --with-1e8 to regenerate it.
Run from the repository root:
    python tests/golden/make_pi_golden.py [--with-1e8]
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.join(ROOT, "tests", "golden", "pi.json")
PI_REF = os.path.join(ROOT, "oracle", "_ref", "pi_ref")

# pi_ref 100000000 --file F: the result of one run of the reference program
# (g++ 13.3 -O3, AVX2 build, x86-64; 2225 s on one core)
RECORDED_1E8 = {"digits": 100000000, "bytes": 100000003,
                "sha256": "80d35f8d6792171abe08f789d6a7815a0c251603426a170df6f59f37748fc474"}


def run(digits):
    with tempfile.TemporaryDirectory() as td:
        f = os.path.join(td, "pi.txt")
        subprocess.run([PI_REF, str(digits), "--file", f], check=True, capture_output=True)
        data = open(f, "rb").read()
    return {"digits": digits, "bytes": len(data), "sha256": hashlib.sha256(data).hexdigest()}


def main():
    subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), "pi"], check=True)
    if not os.path.exists(PI_REF):
        sys.exit("reference sources absent: oracle/_ref/pi_ref not built")
    recs = [run(10 ** e) for e in range(2, 8)]
    recs.append(run(10 ** 8) if "--with-1e8" in sys.argv else RECORDED_1E8)
    with open(OUT, "w") as f:
        json.dump({"generator": "tests/golden/make_pi_golden.py",
                   "program": "preclib pi/pi_chudnovsky.cpp (g++ -O3), output file of `pi_ref DIGITS --file F`",
                   "runs": recs}, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
