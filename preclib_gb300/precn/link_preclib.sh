#!/usr/bin/env bash
# Builds preclib programs with the GPU multiply in place of mul_ntt/mul_fft.
#
#   link_preclib.sh PRECLIB_DIR OUT_DIR PROGRAM.cpp [PROGRAM.cpp ...]
#
# PRECLIB_DIR is preclib's source tree (prec.hpp, src/*.cpp).  Every file of
# src/ is compiled except src/mul_ntt.cpp and src/mul_fft.cpp, whose two
# functions prec_gpu_precn.cpp (beside this script) defines on top of
# libprecgpu.so; each PROGRAM.cpp becomes OUT_DIR/<name> linked against
# that library (run path set).  Built with COUNT_FFTS=1, as preclib's own
# torture and count builds are.  Needs g++ and a built libprecgpu.so.
set -euo pipefail
if [ $# -lt 3 ]; then
  echo "usage: $0 PRECLIB_DIR OUT_DIR PROGRAM.cpp [...]" >&2
  exit 2
fi
SRC=$1
OUT=$2
shift 2
HERE=$(cd "$(dirname "$0")" && pwd)
PKG=$(dirname "$HERE")
ROOT=$(dirname "$PKG")
LIBDIR="$PKG/lib"
if [ ! -f "$SRC/prec.hpp" ]; then
  echo "link_preclib: no prec.hpp under $SRC" >&2
  exit 2
fi
if [ ! -f "$LIBDIR/libprecgpu.so" ]; then
  echo "link_preclib: $LIBDIR/libprecgpu.so missing (python -m preclib_gb300.build)" >&2
  exit 2
fi
mkdir -p "$OUT/obj"
CXX=${CXX:-g++}
FLAGS=(-O3 -std=c++17 -DCOUNT_FFTS=1 -I"$SRC" -I"$ROOT/include")
OBJS=()
pids=()
for f in "$SRC"/src/*.cpp "$HERE/prec_gpu_precn.cpp"; do
  base=$(basename "$f" .cpp)
  case "$base" in mul_ntt|mul_fft) continue ;; esac
  "$CXX" "${FLAGS[@]}" -c "$f" -o "$OUT/obj/$base.o" &
  pids+=($!)
  OBJS+=("$OUT/obj/$base.o")
done
for p in "${pids[@]}"; do wait "$p"; done
for prog in "$@"; do
  name=$(basename "$prog" .cpp)
  "$CXX" "${FLAGS[@]}" "$prog" "${OBJS[@]}" -L"$LIBDIR" -lprecgpu -Wl,-rpath,"$LIBDIR" -o "$OUT/$name"
done
echo "link_preclib: built $* into $OUT"
