#!/bin/bash
# Builds the reference's own GPU kernels (pengdada/SAT integralImage/
# ScanRow-BRLT.cu, BRLT-Scan.cu, ScanRowColumn.cu) for sm_103a into cubins
# under baseline/_ref/ (git-ignored), for the measured reference-GPU baseline
# timed by baseline/ref_gpu_bench.cu.  Test infrastructure, not product code.
#
# SATGB_REF_DIR names the reference checkout's integralImage/ directory.  The
# sources are staged in a scratch directory and given the two compatibility
# changes CUDA 13 needs, nothing else: the legacy unsynchronised warp
# shuffles (__shfl, __shfl_up, ...), removed from CUDA, map to their
# full-warp _sync forms through a header included first, and the expression
# ~uint(31), which no longer parses because `uint` is a macro in the
# reference's cudaLib.cuh, becomes ~31u.  The kernels' algorithms, launch
# shapes and arithmetic are the reference's.  Registers are capped at 64 a
# thread, which the reference's 1024-thread blocks need on this architecture
# (the default allocation asks for more than an SM has for such a block).
set -euo pipefail
: "${SATGB_REF_DIR:?SATGB_REF_DIR must name the integralImage directory of the reference checkout}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
mkdir -p "$OUT"
TMP="$(mktemp -d)"
trap 'rm -rf "$TMP"' EXIT
cp "$SATGB_REF_DIR"/*.cu "$SATGB_REF_DIR"/*.cuh "$SATGB_REF_DIR"/*.h "$TMP"/
sed -i 's/~uint(31)/~31u/g' "$TMP"/*.cu
cat > "$TMP/compat_shfl.h" <<'EOH'
#define __shfl(v, ...) __shfl_sync(0xffffffffu, v, __VA_ARGS__)
#define __shfl_up(v, ...) __shfl_up_sync(0xffffffffu, v, __VA_ARGS__)
#define __shfl_down(v, ...) __shfl_down_sync(0xffffffffu, v, __VA_ARGS__)
#define __shfl_xor(v, ...) __shfl_xor_sync(0xffffffffu, v, __VA_ARGS__)
EOH
NVCC="${NVCC:-nvcc}"
for f in ScanRow-BRLT BRLT-Scan ScanRowColumn; do
  "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -O3 -maxrregcount=64 -w -include "$TMP/compat_shfl.h" -I "$TMP" \
    "$TMP/$f.cu" -o "$OUT/$f.cubin"
done
ls -l "$OUT"/*.cubin
