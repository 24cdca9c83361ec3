#!/usr/bin/env bash
# Stages the reference's kernel sources for the GPU harness (ref_gpu_main.cu).
#
# Test infrastructure only.  The GPU machine has no copy of the reference
# tree, so this copies the reference's own source files, unmodified, from
# PUMP_REFERENCE_DIR (default: the directory "reference" beside the
# repository) into baseline/_ref/src/, which git ignores and which travels
# with the working tree to the GPU machine.  Nothing is committed from it.
set -euo pipefail
HERE=$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)
ROOT=$(cd "$HERE/../.." && pwd)
REF=${PUMP_REFERENCE_DIR:-$(cd "$ROOT/.." && pwd)/reference}
OUT="$ROOT/baseline/_ref/src"
if [ ! -f "$REF/2pBVP.cu" ]; then
  echo "stage_ref.sh: reference sources not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
for f in 2pBVP collisionCheck sampler bvls hsmc PUMP collisionProbability motionPlanningProblem \
         roadMap obstacles; do
  cp "$REF/$f.cu" "$REF/$f.cuh" "$OUT/"
done
cp "$REF/helper.cuh" "$REF/hardCoded.cuh" "$OUT/"
echo "staged the reference kernel sources in $OUT"
