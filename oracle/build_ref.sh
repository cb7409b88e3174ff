#!/usr/bin/env bash
# ORACLE — test infrastructure only.
# Compiles the reference's own CPU collision path, unmodified, into
# oracle/_ref/libref_cpu.so. Sources: the reference checkout named by
# OIBVH_REFERENCE, else the copy stage_ref.sh made under baseline/_ref/oibvh
# (for hosts without the checkout). Needs g++; it does not use the
# reference's CMake build. Flags: -O2 -DNDEBUG (the reference asserts
# on triangle 0, src/cpu/simpleCollide.cpp:91-92, and is built release) and
# -ffp-contract=off (no fused multiply-add, as MSVC's default /fp:precise and
# x86-64 without FMA give the reference's own build).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${OIBVH_REFERENCE:-$(dirname "$HERE")/baseline/_ref/oibvh}"
OUT="$HERE/_ref"
CUDA_INC="${CUDA_HOME:-/usr/local/cuda}/include"
if [ ! -f "$REF/src/cpu/simpleBVH.cpp" ]; then
  echo "reference sources not found under $REF" >&2
  exit 2
fi
mkdir -p "$OUT"
g++ -std=c++17 -O2 -DNDEBUG -ffp-contract=off -fPIC -shared -w \
  -include "$HERE/ref_compat.h" \
  -I"$REF/include" -I"$REF/third" -I"$REF/third/glad/include" -I"$CUDA_INC" \
  "$REF/src/cpu/simpleBVH.cpp" "$REF/src/utils/utils.cpp" "$HERE/ref_harness.cpp" \
  -o "$OUT/libref_cpu.so.tmp"
mv "$OUT/libref_cpu.so.tmp" "$OUT/libref_cpu.so"
echo "built $OUT/libref_cpu.so"

# The reference's GPU kernels (src/cuda/oibvh.cu, src/cuda/collide.cu,
# unmodified, nvcc's default flags as the reference's own build: FMA
# contraction on) with the headless host sequence of ref_gpu_harness.cu, for
# sm_103a, into oracle/_ref/libref_gpu.so. Skipped (with a note) without nvcc.
NVCC="${NVCC:-${CUDA_HOME:-/usr/local/cuda}/bin/nvcc}"
if [ "${OIBVH_REF_GPU:-1}" = "1" ] && [ -x "$NVCC" ]; then
  OBJ="$OUT/gpu_obj"
  mkdir -p "$OBJ"
  NVF=(-gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -w -Xcompiler -fPIC
       -include "$HERE/ref_compat.h" -I"$REF/include" -I"$REF/third" -I"$REF/third/glad/include")
  "$NVCC" "${NVF[@]}" -c "$REF/src/cuda/oibvh.cu" -o "$OBJ/oibvh.o" &
  "$NVCC" "${NVF[@]}" -c "$REF/src/cuda/collide.cu" -o "$OBJ/collide.o" &
  "$NVCC" "${NVF[@]}" -c "$HERE/ref_gpu_harness.cu" -o "$OBJ/harness.o" &
  wait
  "$NVCC" -gencode arch=compute_103a,code=sm_103a -shared -o "$OUT/libref_gpu.so.tmp" \
    "$OBJ/oibvh.o" "$OBJ/collide.o" "$OBJ/harness.o"
  mv "$OUT/libref_gpu.so.tmp" "$OUT/libref_gpu.so"
  echo "built $OUT/libref_gpu.so"
else
  echo "reference GPU kernels not built (no nvcc)"
fi
