#!/bin/sh
# Builds the reference-side test harnesses.  Test infrastructure only.
#
# Where the reference tree is mounted (CMN_REFERENCE, default
# /root/reference), this recipe
#   - compiles oracle/_ref/ref_harness and oracle/_ref/ref_gams from the
#     reference's own host sources, where they lie, for this machine (they
#     generate the golden fixtures under tests/golden/);
#   - writes oracle/_ref/cuminlp_ref_gpu.cuh, the reference's headers for its
#     SearchDriver, policies, AggregateDriver, GAMS frontend interface and
#     CUDA graph backend as one file, and oracle/_ref/cuminlp_ref_gams.cpp,
#     its GAMS frontend source with its headers (oracle/amalgamate.py); and
#     copies the reference's test models (test/data/gams) to
#     oracle/_ref/gams.  All of it travels with the working tree to the GPU
#     host, where oracle/build.py compiles oracle/ref_gpu.cu against it.
# Without the reference tree it does nothing and exits 0.
#
# The reference's device code contracts `a + b*c` into FMA (nvcc's default);
# -mfma -ffp-contract=fast gives its host code (region/decode.hpp) the same
# contraction, so the decoded boxes are the ones the reference's GPU backend
# evaluates.  The host harnesses are x86-64 only, like this container.
set -eu
REF=${CMN_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/include/cuminlp" ]; then
  echo "reference tree not found at $REF; nothing to build"
  exit 0
fi
mkdir -p "$OUT"
PY=${PYTHON:-python3}
"$PY" "$HERE/amalgamate.py" "$REF" "$OUT/cuminlp_ref_gpu.cuh" \
  include/cuminlp/search/driver.hpp include/cuminlp/policy/greedy_enum.hpp \
  include/cuminlp/policy/width_first.hpp include/cuminlp/policy/bisection_budget.hpp \
  include/cuminlp/aggregate/driver.hpp include/cuminlp/gams.hpp \
  include/cuminlp/backend/graph/factory.cuh
# the GAMS frontend (a source file with its own headers), and the reference's
# MINLPLib test models it is tested on
"$PY" "$HERE/amalgamate.py" "$REF" "$OUT/cuminlp_ref_gams.cpp" source/gams/frontend.cpp
mkdir -p "$OUT/gams"
cp "$REF"/test/data/gams/*.gms "$OUT/gams/"
case "$(uname -m)" in
  x86_64) ;;
  *) echo "host harnesses are built on x86-64 only"; exit 0 ;;
esac
CC=${CC:-gcc}
CXX=${CXX:-g++}
"$CC" -O2 -std=c11 -ffp-contract=off -fPIC -c "$HERE/oracle.c" -o "$OUT/oracle.o"
"$CXX" -O2 -std=c++20 -mfma -ffp-contract=fast -I"$HERE/ref_shim" -I"$REF/include" -I"$HERE" \
  "$HERE/ref_harness.cpp" "$OUT/oracle.o" -o "$OUT/ref_harness" -lm -lpthread
# the reference's GAMS frontend, without contraction (its constant folding is
# plain IEEE arithmetic on the host)
"$CXX" -O2 -std=c++20 -ffp-contract=off -I"$HERE/ref_shim" -I"$REF/include" -I"$REF/source/gams" \
  "$REF/source/gams/frontend.cpp" "$HERE/ref_gams.cpp" -o "$OUT/ref_gams" -lm
echo "$OUT/ref_harness $OUT/ref_gams $OUT/cuminlp_ref_gpu.cuh"
