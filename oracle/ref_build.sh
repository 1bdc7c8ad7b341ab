#!/usr/bin/env bash
# Builds the checker pieces of the reference from its own sources (where they lie under
# the reference checkout) into oracle/_ref/: its grid index code, its MMA solver, and
# its CUDA solver path run on the host through oracle/ref_emu (a CUDA runtime, cuBLAS and
# cuSOLVER stand-in that executes the reference kernels on the CPU).
#   usage: oracle/ref_build.sh [REFERENCE_ROOT]
#   (default: $STOKES_TO_REFERENCE, else the checkout this build container mounts)
set -euo pipefail
REF="${1:-${STOKES_TO_REFERENCE:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
CC_DIR="$REF/simplex/src/common_cpx"
if [ ! -f "$CC_DIR/grid3D.cu" ]; then
  echo "reference sources not found under $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
NVCC="${NVCC:-nvcc}"
"$NVCC" -std=c++14 -O2 -Xcompiler -fPIC -shared -gencode arch=compute_103a,code=sm_103a \
  -I "$CC_DIR" "$HERE/ref_grid3d_wrap.cu" "$CC_DIR/grid3D.cu" -o "$OUT/libref_grid3d.so"
echo "built $OUT/libref_grid3d.so"
# grid2D lives in form01mapping.cu beside the 2D mapping kernels (extended lambdas, gpuUtils)
"$NVCC" -std=c++14 -O2 -Xcompiler -fPIC -shared --extended-lambda -w -gencode arch=compute_103a,code=sm_103a \
  -I "$CC_DIR" "$HERE/ref_grid2d_wrap.cu" "$CC_DIR/form01mapping.cu" "$CC_DIR/gpuUtils.cu" -o "$OUT/libref_grid2d.so" -lcublas
echo "built $OUT/libref_grid2d.so"
# the vendored MMA solver (plain C++, no dependencies)
MMA_DIR="$REF/simplex/ext/mma"
"${CXX:-g++}" -std=c++14 -O2 -fPIC -shared -w -I "$MMA_DIR" "$HERE/ref_mma_wrap.cpp" "$MMA_DIR/MMASolver.cpp" \
  -o "$OUT/libref_mma.so"
echo "built $OUT/libref_mma.so"
# the reference's CUDA solver path (3D and 2D), run on the host through the CUDA stand-in
"${PYTHON:-python3}" "$HERE/ref_emu/build.py" "$REF"
