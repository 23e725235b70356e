#!/usr/bin/env bash
# Builds the reference's own CPU brute-force join (brute_force in
# src/utils.cu:285-317 of bwd29/self-join-MiSTIC) from its unmodified source
# where it lies, plus oracle/ref_driver.cpp, into oracle/_ref/ref_brute; and
# its text -> binary converter (toCSV.cpp, the `toBin` tool) into
# oracle/_ref/ref_tobin.
# Only this recipe reads the reference tree; outputs go to oracle/_ref/ only.
# The reference headers need BS/KB defined (include/params.cuh) and thrust,
# so the file is compiled with nvcc as host code; no GPU is touched.
# Usage: oracle/build_ref.sh [reference_root]
#   reference_root: the first argument, else $MISTIC_REFERENCE_ROOT, else a
#   checkout named `reference` beside this repository.  Where none exists the
#   recipe does nothing (the GPU machines have no reference tree).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF=${1:-${MISTIC_REFERENCE_ROOT:-$HERE/../../reference}}
OUT="$HERE/_ref"
if [ ! -f "$REF/src/utils.cu" ]; then
  echo "reference source not found at $REF; nothing to build" >&2
  exit 0
fi
mkdir -p "$OUT"
nvcc -O3 -DBS=256 -DKB=1024 -DDIM=18 -I"$REF" -Xcompiler -fopenmp \
     -Xcompiler -ffp-contract=off \
     -c "$REF/src/utils.cu" -o "$OUT/ref_utils.o"
g++ -O2 -fopenmp -c "$HERE/ref_driver.cpp" -o "$OUT/ref_driver.o"
nvcc -Xcompiler -fopenmp "$OUT/ref_driver.o" "$OUT/ref_utils.o" -o "$OUT/ref_brute"
echo "built $OUT/ref_brute"
if [ -f "$REF/toCSV.cpp" ]; then
  g++ -O2 "$REF/toCSV.cpp" -o "$OUT/ref_tobin"
  echo "built $OUT/ref_tobin"
fi
