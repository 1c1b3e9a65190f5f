#!/usr/bin/env bash
# Build the reference's own multiply from its sources into oracle/_ref/.
# TEST INFRASTRUCTURE ONLY: used to pin the C restatement and to generate
# golden vectors.  Needs the reference tree (default /root/reference); does
# nothing and exits 0 when it is absent.  Outputs go only to oracle/_ref/.
#   libprecref.so       portable build (-O3, no SIMD flags), COUNT_FFTS on
#   libprecref_avx2.so  x86-64 only: -mavx2 build, for the CPU-baseline table
#   pi_ref              (argument "pi") preclib's pi program, for golden hashes
#   interposed/         (argument "interposed") preclib's fft_torture,
#                       test_opt_smoke and pi_chudnovsky linked with the GPU
#                       mul_ntt / mul_fft instead of src/mul_ntt.cpp, mul_fft.cpp
set -euo pipefail
REF=${PRECLIB_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/prec.hpp" ]; then
  echo "build_ref: reference sources not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
if [ "${1:-}" = "pi" ]; then
  # preclib's own pi program (its CPU multiply), for the golden digit hashes
  "${CXX:-g++}" -O3 -std=c++17 -I"$REF" "$REF/pi/pi_chudnovsky.cpp" "$REF"/src/*.cpp -o "$OUT/pi_ref.tmp"
  mv "$OUT/pi_ref.tmp" "$OUT/pi_ref"
  exit 0
fi
if [ "${1:-}" = "interposed" ]; then
  # preclib's own programs with mul_ntt/mul_fft from the GPU library
  # (needs preclib_gb300/lib/libprecgpu.so built first)
  "$HERE/../preclib_gb300/precn/link_preclib.sh" "$REF" "$OUT/interposed" \
    "$REF/test/fft_torture.cpp" "$REF/test/test_opt_smoke.cpp" "$REF/pi/pi_chudnovsky.cpp"
  exit 0
fi
CXX=${CXX:-g++}
SRCS=("$REF"/src/*.cpp)
"$CXX" -O3 -std=c++17 -fPIC -shared -DCOUNT_FFTS=1 -I"$REF" \
  "$HERE/ref_shim.cpp" "${SRCS[@]}" -o "$OUT/libprecref.so.tmp"
mv "$OUT/libprecref.so.tmp" "$OUT/libprecref.so"
if [ "$(uname -m)" = "x86_64" ]; then
  "$CXX" -O3 -mavx2 -std=c++17 -fPIC -shared -DCOUNT_FFTS=1 -I"$REF" \
    "$HERE/ref_shim.cpp" "${SRCS[@]}" -o "$OUT/libprecref_avx2.so.tmp"
  mv "$OUT/libprecref_avx2.so.tmp" "$OUT/libprecref_avx2.so"
fi
echo "build_ref: built $OUT"
