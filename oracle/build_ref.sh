#!/usr/bin/env bash
# Build the reference's own host-compilable functors into oracle/_ref/.
#   usage: build_ref.sh <output dir> [<reference root>]
# The reference root defaults to where this container keeps the reference's
# sources; without them the script does nothing (the GPU hosts never have
# them).  The reference's CUDA file is compiled where it lies (included by
# ref/harness.cpp) with g++ on Thrust's CPP backend; ref/shim.h supplies
# what the 2012 code base expects from its toolchain.  Nothing is copied.
set -euo pipefail
OUT="$1"; REF="${2:-/root/reference}"
[ -d "$REF/tau_leaping" ] || exit 0
HERE="$(cd "$(dirname "$0")" && pwd)"
CUDA_INC=/usr/local/cuda/include
mkdir -p "$OUT"
if [ ! -f "$OUT/libtlref.so" ] || [ "$HERE/ref/harness.cpp" -nt "$OUT/libtlref.so" ] || [ "$HERE/ref/shim.h" -nt "$OUT/libtlref.so" ]; then
  g++ -std=c++17 -O1 -fPIC -shared -w -DNDEBUG \
    -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP -D__global__= \
    -I"$REF" -I"$REF/tau_leaping" -I"$CUDA_INC" -I"$CUDA_INC/cccl" \
    -include "$HERE/ref/shim.h" \
    "$HERE/ref/harness.cpp" -o "$OUT/libtlref.so"
  echo "built $OUT/libtlref.so"
fi

# The reference's whole host path + a driver with logging on -> ref_driver.
DRV="$OUT/ref_driver"
if [ ! -f "$DRV" ] || [ "$HERE/ref/driver.cpp" -nt "$DRV" ] || [ "$HERE/ref/shim_full.h" -nt "$DRV" ] || [ "$HERE/ref/stubs.cpp" -nt "$DRV" ]; then
  OBJ="$OUT/obj"; mkdir -p "$OBJ"
  FLAGS="-std=c++17 -O2 -w -DNDEBUG -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP -D__global__= -I$REF -I$REF/tau_leaping -I$CUDA_INC -I$CUDA_INC/cccl -include $HERE/ref/shim_full.h"
  pids=()
  for src in model.cu model.cpp ModelConst.cu ModelState.cu CSRMatrixPacked.cu CSRMatrix.cu CSCMatrix.cu \
             CSCHostMatrixData.cpp StochKitReader.cpp functions.cpp statistics.cpp; do
    g++ $FLAGS -x c++ -c "$REF/tau_leaping/$src" -o "$OBJ/${src}.o" & pids+=($!)
  done
  g++ $FLAGS -x c++ -c "$HERE/ref/driver.cpp" -o "$OBJ/driver.o" & pids+=($!)
  g++ -std=c++17 -O2 -w -I$CUDA_INC -c "$HERE/ref/stubs.cpp" -o "$OBJ/stubs.o" & pids+=($!)
  for p in "${pids[@]}"; do wait "$p"; done
  g++ -o "$DRV" "$OBJ"/*.o
  echo "built $DRV"
fi
