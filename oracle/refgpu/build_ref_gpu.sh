#!/usr/bin/env bash
# Builds ref_gpu_N<N>: the reference's own kernel sources (staged in
# baseline/_ref/src by stage_ref.sh) compiled by nvcc as the reference's
# Makefile compiles them (-O3 -rdc=true, nvcc's default contraction; the
# Makefile's -arch=sm_52 becomes sm_103a, which CUDA 13 supports), linked with
# the harness main (ref_gpu_main.cu), the two helper stand-ins of
# oracle/refcpu/ref_helpers.cpp and the particle tables of
# oracle/refcpu/ref_support.cpp.  Host code of the harness and the tables is
# compiled without contraction, so the tables are bit-identical on every
# host.  Output: oracle/_ref/ref_gpu_N<N> (git-ignored).
#
# Test infrastructure only; runs on the GPU machine (nvcc, no GPU needed).
set -euo pipefail
HERE=$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)
ROOT=$(cd "$HERE/../.." && pwd)
SRC="$ROOT/baseline/_ref/src"
OUT="$ROOT/oracle/_ref"
NUMS=${PUMPREF_NUMS:-"1000 4000"}
CUDA_HOME=${CUDA_HOME:-/usr/local/cuda}
NVCC="$CUDA_HOME/bin/nvcc"
if [ ! -f "$SRC/2pBVP.cu" ]; then
  echo "build_ref_gpu.sh: no staged reference sources in $SRC (run stage_ref.sh where the reference is)" >&2
  exit 1
fi
mkdir -p "$OUT"
TMP=$(mktemp -d)
trap 'rm -rf "$TMP"' EXIT
ARCH="-gencode arch=compute_103a,code=sm_103a"
HOSTFP="-Xcompiler -ffp-contract=off,-fno-fast-math"
gcc -O2 -ffp-contract=off -fno-fast-math -c "$ROOT/oracle/pump_oracle.c" -o "$TMP/pump_oracle.o"
g++ -O2 -ffp-contract=off -fno-fast-math -c "$ROOT/oracle/refcpu/ref_support.cpp" -o "$TMP/ref_support.o"
g++ -O2 -c "$ROOT/oracle/refcpu/ref_helpers.cpp" -o "$TMP/ref_helpers.o"
build_one() {
  local N=$1
  local D="$TMP/N$N"
  mkdir -p "$D"
  local objs=()
  for f in 2pBVP collisionCheck sampler bvls hsmc PUMP collisionProbability motionPlanningProblem \
           roadMap obstacles; do
    "$NVCC" -O3 -rdc=true $ARCH -DDIM=6 -DNUM=$N -w -I"$SRC" -c "$SRC/$f.cu" -o "$D/$f.o"
    objs+=("$D/$f.o")
  done
  "$NVCC" -O3 -rdc=true $ARCH $HOSTFP -DDIM=6 -DNUM=$N -I"$SRC" -c "$HERE/ref_gpu_main.cu" -o "$D/main.o"
  "$NVCC" -rdc=true $ARCH "${objs[@]}" "$D/main.o" "$TMP/pump_oracle.o" "$TMP/ref_support.o" \
    "$TMP/ref_helpers.o" -o "$OUT/ref_gpu_N$N"
  echo "built $OUT/ref_gpu_N$N"
}
pids=()
for N in $NUMS; do build_one "$N" & pids+=($!); done
for p in "${pids[@]}"; do wait "$p"; done
