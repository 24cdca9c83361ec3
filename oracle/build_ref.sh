#!/usr/bin/env bash
# Builds the reference PUMP program for the CPU, as the parity oracle.
#
# Test infrastructure only.  Reads the reference sources where they lie
# (PUMP_REFERENCE_DIR, default: the directory "reference" beside the
# repository) and writes only into
# oracle/_ref/ (git-ignored).  For each sample count N in PUMPREF_NUMS the
# reference's NUM is a compile-time constant (Makefile:1-5), so one pair of
# artefacts is built per N:
#
#   libpumpref_cpu_N<N>.so  the reference's kernel sources (2pBVP.cu,
#                           collisionCheck.cu, sampler.cu, bvls.cu, hsmc.cu,
#                           PUMP.cu, collisionProbability.cu) compiled by g++
#                           as host C++ through refcpu/shim.h, plus the CPU
#                           launcher (refcpu/launcher.cpp).  g++ cannot parse
#                           the `<<<grid, block>>>` launch syntax, so the two
#                           files that mix launches with kernels are passed
#                           through a one-line sed that deletes the launch
#                           configuration into a temporary directory outside
#                           the repository; the launch sites sit in host
#                           functions this library never calls.
#   pump_ref_N<N>           the reference's own main() and host code
#                           (mainPUMP.cu, PUMP.cu, ...) through nvcc's host
#                           pass, with Thrust replaced by refcpu/stub_thrust, linked
#                           against refcpu/fake_cudart.cpp.
#
# Both use refcpu/ipow.cpp (correctly rounded integer powers) and never
# contract multiply-adds, which is the arithmetic the library and the C
# oracle implement.  Nothing here is needed at run time on a GPU machine.
#
# An entry N:P of PUMPREF_NUMS builds the program with the reference's HSMC
# particle count numHSMCParticles (a const int, mainPUMP.cu:68, 128 in the
# tree) set to P: a copy of mainPUMP.cu with that one line changed is put in
# a temporary directory searched before the reference tree.  The artefacts
# are then named pump_ref_N<N>_P<P> / libpumpref_cpu_N<N>_P<P>.so.
set -euo pipefail
HERE=$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)
REF=${PUMP_REFERENCE_DIR:-$(cd "$HERE/../.." && pwd)/reference}
OUT="$HERE/_ref"
NUMS=${PUMPREF_NUMS:-"64 1000"}
CUDA_HOME=${CUDA_HOME:-/usr/local/cuda}
NVCC="$CUDA_HOME/bin/nvcc"

if [ ! -f "$REF/mainPUMP.cu" ]; then
  echo "build_ref.sh: reference sources not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
TMP=$(mktemp -d)
trap 'rm -rf "$TMP"' EXIT

FP="-ffp-contract=off -fno-fast-math"
g++ -O2 $FP -fPIC -c "$HERE/refcpu/ipow.cpp" -o "$TMP/ipow.o"
gcc -O2 $FP -fPIC -fopenmp -c "$HERE/pump_oracle.c" -o "$TMP/pump_oracle.o"
g++ -O2 $FP -c "$HERE/refcpu/ref_support.cpp" -o "$TMP/ref_support.o"
g++ -O2 $FP -fPIC -c "$HERE/refcpu/ref_helpers.cpp" -o "$TMP/ref_helpers.o"

sed 's/<<<[^>]*>>>//' "$REF/PUMP.cu" > "$TMP/PUMP.cu"
sed 's/<<<[^>]*>>>//' "$REF/collisionProbability.cu" > "$TMP/collisionProbability.cu"

for NP in $NUMS; do
  N=${NP%%:*}
  P=${NP#*:}
  TAG=N$N
  INC=()
  if [ "$P" != "$NP" ] && [ "$P" != 128 ]; then
    TAG=N${N}_P$P
    mkdir -p "$TMP/$TAG"
    sed "s/^const int numHSMCParticles = 128;/const int numHSMCParticles = $P;/" "$REF/mainPUMP.cu" \
      > "$TMP/$TAG/mainPUMP.cu"
    grep -q "^const int numHSMCParticles = $P;" "$TMP/$TAG/mainPUMP.cu"
    INC=(-I"$TMP/$TAG")
  fi
  DEFS="-DDIM=6 -DNUM=$N"
  # CPU kernel library (reference kernels as host C++)
  g++ -O2 $FP -fPIC -shared -fopenmp -w -Wl,-Bsymbolic \
    -include "$HERE/refcpu/shim.h" -I"$HERE/refcpu/stub_cuda" -I"$HERE/refcpu/stub_thrust" -I"$REF" $DEFS \
    -x c++ "$REF/2pBVP.cu" "$REF/collisionCheck.cu" "$REF/sampler.cu" "$REF/bvls.cu" \
    "$REF/hsmc.cu" "$TMP/PUMP.cu" "$TMP/collisionProbability.cu" \
    "$HERE/refcpu/launcher.cpp" -x none "$TMP/ipow.o" "$TMP/ref_helpers.o" \
    -o "$OUT/libpumpref_cpu_$TAG.so"
  # reference program: nvcc host pass over the unmodified sources
  "$NVCC" -cuda -x cu "$HERE/refcpu/ref_all.cu" -I"$HERE/refcpu/stub_thrust" "${INC[@]}" -I"$REF" $DEFS \
    -O3 -w -gencode arch=compute_103a,code=sm_103a -o "$TMP/ref_all_$TAG.cpp.ii"
  g++ -O2 $FP -w -c -x c++ "$TMP/ref_all_$TAG.cpp.ii" -o "$TMP/ref_all_$TAG.o"
  g++ -O2 $FP $DEFS -I"$CUDA_HOME/include" -c "$HERE/refcpu/fake_cudart.cpp" -o "$TMP/fake_cudart_$TAG.o"
  g++ -o "$OUT/pump_ref_$TAG" "$TMP/ref_all_$TAG.o" "$TMP/fake_cudart_$TAG.o" "$TMP/ref_support.o" \
    "$TMP/ipow.o" "$TMP/ref_helpers.o" "$TMP/pump_oracle.o" -ldl -fopenmp
  echo "built $OUT/pump_ref_$TAG and $OUT/libpumpref_cpu_$TAG.so"
done
