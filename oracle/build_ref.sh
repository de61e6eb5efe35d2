#!/bin/sh
# Builds oracle/_ref/libnbfmm_refcpu.so: the reference's kernelFunction and vector operators compiled for the
# CPU from the reference headers where they lie (see oracle/ref_shim.cpp). Test infrastructure only.
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
${CXX:-g++} -O2 -ffp-contract=off -fPIC -shared \
  -I"$here/_ref/include" -I"$ref/include" -I"$cuda/include" \
  "$here/ref_shim.cpp" -o "$here/_ref/libnbfmm_refcpu.so"
echo "build_ref: wrote $here/_ref/libnbfmm_refcpu.so"
