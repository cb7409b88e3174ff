#!/usr/bin/env bash
# ORACLE — test infrastructure only.
# Copies the reference sources that its CPU collision path (and its GPU
# kernels) compile from into baseline/_ref/oibvh/, which is git-ignored and
# travels with the working tree to hosts that have no reference checkout, so
# that build_ref.sh can compile the reference natively there (an x86 build does
# not run on an Arm host). Needs OIBVH_REFERENCE: the reference checkout.
# Nothing under baseline/_ref/ is committed.
set -euo pipefail
REF="${OIBVH_REFERENCE:?set OIBVH_REFERENCE to the reference checkout}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
DST="$(dirname "$HERE")/baseline/_ref/oibvh"
if [ ! -f "$REF/src/cpu/simpleBVH.cpp" ]; then
  echo "reference sources not found under $REF" >&2
  exit 2
fi
rm -rf "$DST.tmp"
mkdir -p "$DST.tmp/src/cpu" "$DST.tmp/src/utils" "$DST.tmp/src/cuda" "$DST.tmp/third/glad"
cp "$REF/src/cpu/simpleBVH.cpp" "$DST.tmp/src/cpu/"
cp "$REF/src/utils/utils.cpp" "$DST.tmp/src/utils/"
cp "$REF/src/cuda/oibvh.cu" "$REF/src/cuda/collide.cu" "$DST.tmp/src/cuda/"
cp -r "$REF/include" "$DST.tmp/include"
cp -r "$REF/third/glm" "$REF/third/gProximity" "$DST.tmp/third/"
cp -r "$REF/third/glad/include" "$DST.tmp/third/glad/include"
rm -rf "$DST"
mv "$DST.tmp" "$DST"
echo "staged $DST"
