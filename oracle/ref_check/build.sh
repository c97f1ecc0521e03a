#!/bin/sh
# Builds oracle/_ref/libfv2d_ref.so from the reference's own headers, compiled
# in place from REF_DIR (default: baseline/_ref, where oracle/ref_check/stage.sh
# puts them) against the serial stand-ins in oracle/ref_check/include.  Test
# infrastructure only: used to pin the oracle, to generate the fixtures under
# tests/golden/ and to time the reference's own step code on the host cores.
# Outputs go to oracle/_ref/ only.  Exits 2 when REF_DIR holds no reference.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_DIR="${REF_DIR:-$HERE/../../baseline/_ref}"
OUT="$HERE/../_ref"
[ -f "$REF_DIR/Update.h" ] || { echo "reference sources not found at $REF_DIR" >&2; exit 2; }
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
