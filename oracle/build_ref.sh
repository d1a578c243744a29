#!/bin/sh
# Builds oracle/_ref/libref.so from the reference's own sources where they lie
# (REF_DIR; this recipe is the one place that knows their default location),
# plus the small shims in oracle/ref/.  Exits 0 without building when the
# sources are absent.
# The reference's kernel file is compiled as plain C++ against a host
# stand-in for the CUDA headers so its kernel bodies run on the CPU.
# Used only to pin the oracle; the output stays out of git.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF_DIR=${REF_DIR:-/root/reference}
OUT="$HERE/_ref"
if [ ! -f "$REF_DIR/trove_functions.cpp" ]; then
  exit 0
fi
mkdir -p "$OUT"
CXX=${CXX:-g++}
FLAGS="-O2 -fPIC -ffp-contract=off -std=c++11 -w -I$HERE/ref/inc -I$REF_DIR"
$CXX $FLAGS -c -x c++ "$REF_DIR/dipole_kernals.cu" -o "$OUT/dipole_kernals.o"
$CXX $FLAGS -c "$REF_DIR/trove_functions.cpp" -o "$OUT/trove_functions.o"
$CXX $FLAGS -c "$HERE/ref/util_shim.cpp" -o "$OUT/util_shim.o"
$CXX $FLAGS -std=c++17 -c "$HERE/ref/ref_wrap.cpp" -o "$OUT/ref_wrap.o"
$CXX -shared -o "$OUT/libref.so" "$OUT/dipole_kernals.o" "$OUT/trove_functions.o" \
    "$OUT/util_shim.o" "$OUT/ref_wrap.o"
rm -f "$OUT"/*.o
echo "built $OUT/libref.so"
