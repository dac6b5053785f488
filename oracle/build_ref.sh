#!/bin/sh
# Builds oracle/_ref/ref_harness from the reference's own sources, where they
# lie, plus the CPU oracle.  Test infrastructure only; run in the container
# that mounts the reference (the GPU host has no reference tree).
#
# The reference's device code contracts `a + b*c` into FMA (nvcc's default);
# -mfma -ffp-contract=fast gives its host code (region/decode.hpp) the same
# contraction, so the decoded boxes are the ones the reference's GPU backend
# evaluates.  x86-64 only, like this container.
set -eu
REF=${REF:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
mkdir -p "$OUT"
CC=${CC:-gcc}
CXX=${CXX:-g++}
"$CC" -O2 -std=c11 -ffp-contract=off -fPIC -c "$HERE/oracle.c" -o "$OUT/oracle.o"
"$CXX" -O2 -std=c++20 -mfma -ffp-contract=fast -I"$HERE/ref_shim" -I"$REF/include" -I"$HERE" \
  "$HERE/ref_harness.cpp" "$OUT/oracle.o" -o "$OUT/ref_harness" -lm -lpthread
# the reference's GAMS frontend, without contraction (its constant folding is
# plain IEEE arithmetic on the host)
"$CXX" -O2 -std=c++20 -ffp-contract=off -I"$HERE/ref_shim" -I"$REF/include" -I"$REF/source/gams" \
  "$REF/source/gams/frontend.cpp" "$HERE/ref_gams.cpp" -o "$OUT/ref_gams" -lm
echo "$OUT/ref_harness $OUT/ref_gams"
