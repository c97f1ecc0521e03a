#!/bin/sh
# Builds oracle/_ref/libfv2d_ref.so from the reference's own headers, compiled
# in place from the reference checkout (REF_DIR, default /root/reference)
# against the serial stand-ins in oracle/ref_check/include.  Test
# infrastructure only: used to pin the oracle and to generate the fixtures
# under tests/golden/.  Outputs go to oracle/_ref/ only.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_DIR="${REF_DIR:-/root/reference}"
OUT="$HERE/../_ref"
[ -f "$REF_DIR/Update.h" ] || { echo "reference checkout not found at $REF_DIR" >&2; exit 2; }
mkdir -p "$OUT"
${CXX:-g++} -std=c++20 -O2 -ffp-contract=off -fPIC -shared -w \
  -I"$HERE/include" -I"$REF_DIR" \
  -o "$OUT/libfv2d_ref.so" "$HERE/ref_harness.cpp"
echo "built $OUT/libfv2d_ref.so"
# the same sources with OpenMP over rows (a release-style build of the
# reference's step code for timing it on the host cores)
${CXX:-g++} -std=c++20 -O3 -fopenmp -ffp-contract=off -fPIC -shared -w \
  -I"$HERE/include" -I"$REF_DIR" \
  -o "$OUT/libfv2d_ref_omp.so" "$HERE/ref_harness.cpp"
echo "built $OUT/libfv2d_ref_omp.so"
