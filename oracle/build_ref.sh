#!/bin/sh
# Builds oracle/_ref/libnbfmm_refcpu.so: the reference's kernelFunction and vector operators compiled for the
# CPU from the reference headers where they lie, and its frame raster kernel displayDevice
# (source/nbfmm/display/stars/display.cu:29-214), which is cut out of that file into oracle/_ref/ as a build
# intermediate because the rest of the file needs nvcc (see oracle/ref_shim.cpp). Test infrastructure only.
# The reference's config.hpp is generated by its CMake; the two headers used here only need it to exist,
# so an empty stand-in is written under oracle/_ref/include.
set -eu
here=$(cd "$(dirname "$0")" && pwd)
ref=${NBFMM_REFERENCE:-/root/reference}
cuda=${CUDA_HOME:-/usr/local/cuda}
if [ ! -f "$ref/include/nbfmm/core/kernel_function.hpp" ]; then
  echo "build_ref: reference sources not found at $ref; skipped" >&2
  exit 0
fi
mkdir -p "$here/_ref/include/nbfmm"
printf '#pragma once\n' > "$here/_ref/include/nbfmm/config.hpp"
defs=""
disp="$ref/source/nbfmm/display/stars/display.cu"
if [ -f "$disp" ]; then
  sed -n '/^__global__ void displayDevice(/,/^}/p' "$disp" > "$here/_ref/display_device.inc"
  if grep -q '^}' "$here/_ref/display_device.inc"; then defs="-DNBFMM_REF_DISPLAY"; fi
fi
${CXX:-g++} -O2 -ffp-contract=off -fPIC -shared $defs \
  -I"$here/_ref" -I"$here/_ref/include" -I"$ref/include" -I"$cuda/include" \
  "$here/ref_shim.cpp" -o "$here/_ref/libnbfmm_refcpu.so"
echo "build_ref: wrote $here/_ref/libnbfmm_refcpu.so"
