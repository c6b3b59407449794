#!/usr/bin/env bash
# Build the reference's own host-compilable functors into oracle/_ref/.
#   usage: build_ref.sh <reference root> <output dir>
# The reference's CUDA file is compiled where it lies (included by
# ref/harness.cpp) with g++ on Thrust's CPP backend; ref/shim.h supplies
# what the 2012 code base expects from its toolchain.  Nothing is copied.
set -euo pipefail
REF="$1"; OUT="$2"
HERE="$(cd "$(dirname "$0")" && pwd)"
CUDA_INC=/usr/local/cuda/include
mkdir -p "$OUT"
if [ -f "$OUT/libtlref.so" ] && [ "$OUT/libtlref.so" -nt "$HERE/ref/harness.cpp" ] && [ "$OUT/libtlref.so" -nt "$HERE/ref/shim.h" ]; then
  exit 0
fi
g++ -std=c++17 -O1 -fPIC -shared -w -DNDEBUG \
  -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP -D__global__= \
  -I"$REF" -I"$REF/tau_leaping" -I"$CUDA_INC" -I"$CUDA_INC/cccl" \
  -include "$HERE/ref/shim.h" \
  "$HERE/ref/harness.cpp" -o "$OUT/libtlref.so"
echo "built $OUT/libtlref.so"
