#!/usr/bin/env bash
# Builds the reference's own GPU join -- build/main of bwd29/self-join-MiSTIC,
# src/{main,launcher,kernel,nodes,tree,utils}.cu, unmodified -- for sm_103a,
# one binary per dimensionality (the reference fixes DIM at compile time,
# Makefile:16; BS=256 and KB=1024 as script.sh builds it) into
# oracle/_ref/ref_main_d<DIM>.  It is timed beside the library and its
# "Total results Set Size" is compared with the oracle's count; nothing of it
# enters the library.
#
# The reference hard-codes CUDA_DEVICE 1 (include/params.cuh:40); on a
# one-GPU machine cudaSetDevice(1) fails and thrust then reports "invalid
# device ordinal".  The sources are compiled with cudaSetDevice renamed to
# mistic_ref_set_device (oracle/ref_device_shim.cpp), which selects device 0;
# no source line is changed.
#
# The GPU machines have no reference tree and run no binary built here, so
# where the tree is present (argument 1, $MISTIC_REFERENCE_ROOT, or a checkout
# named `reference` beside this repository) the recipe stages its src/ and
# include/ into oracle/_ref/gpu_src (git-ignored: never part of this
# repository's history, only carried with the working copy to the machine
# that builds it); where only the staged copy exists it builds from that.
# Usage: oracle/build_ref_gpu.sh [reference_root] [DIM ...]   (default DIMs: 18 90)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF=${1:-${MISTIC_REFERENCE_ROOT:-$HERE/../../reference}}
shift || true
DIMS=${*:-"18 90"}
OUT="$HERE/_ref"
SRC="$OUT/gpu_src"
mkdir -p "$OUT"
if [ -f "$REF/src/launcher.cu" ]; then
  rm -rf "$SRC"
  mkdir -p "$SRC"
  cp -r "$REF/src" "$REF/include" "$SRC/"
  chmod -R u+w "$SRC"
fi
if [ ! -f "$SRC/src/launcher.cu" ]; then
  echo "no reference GPU source (tree or staged copy); nothing to build" >&2
  exit 0
fi
command -v nvcc >/dev/null || { echo "nvcc not found" >&2; exit 1; }
FLAGS="-O3 -gencode arch=compute_103a,code=sm_103a -Xcompiler -fopenmp -DBS=256 -DKB=1024 -I$SRC -DcudaSetDevice=mistic_ref_set_device"
for D in $DIMS; do
  B="$OUT/build_d$D"
  mkdir -p "$B"
  pids=()
  for f in main launcher kernel nodes tree utils; do
    nvcc $FLAGS -DDIM="$D" -c "$SRC/src/$f.cu" -o "$B/$f.o" > "$B/$f.log" 2>&1 &
    pids+=($!)
  done
  nvcc -O2 -c "$HERE/ref_device_shim.cpp" -o "$B/shim.o" &
  pids+=($!)
  for p in "${pids[@]}"; do wait "$p"; done
  nvcc -gencode arch=compute_103a,code=sm_103a -Xcompiler -fopenmp "$B"/*.o -o "$OUT/ref_main_d$D" -lcuda
  echo "built $OUT/ref_main_d$D"
done
