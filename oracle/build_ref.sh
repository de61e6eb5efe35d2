#!/bin/sh
# Builds oracle/_ref/libnbfmm_refcpu.so: the reference's kernelFunction and vector operators compiled for the
# CPU from the reference headers where they lie, and kernels cut out of their files into oracle/_ref/ as build
# intermediates (the rest of those files needs nvcc; see oracle/ref_shim.cpp): the frame raster displayDevice
# (source/nbfmm/display/stars/display.cu:29-214), Stars::prune's pruneDevice (prune.cu:28-42) and the model
# generators' generate*Device kernels (source/nbfmm/model/*.cu). Test infrastructure only.
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
# Stars::prune's flag kernel (source/nbfmm/display/stars/prune.cu:28-42); its thrust::sort_by_key runs on
# thrust's host (CPP) system in ref_shim.cpp.
prune="$ref/source/nbfmm/display/stars/prune.cu"
if [ -f "$prune" ]; then
  sed -n '/^__global__ void pruneDevice(/,/^}/p' "$prune" > "$here/_ref/prune_device.inc"
  if grep -q '^}' "$here/_ref/prune_device.inc"; then defs="$defs -DNBFMM_REF_PRUNE"; fi
fi
# The model generators' kernels (source/nbfmm/model/*.cu, generate*Device) and, for the two circle models, the
# two host lines that compute the angle step passed to the kernel.
models=1
for m in circle_center circle_uniform_center disk disk_center disk_static rectangle; do
  f="$ref/source/nbfmm/model/$m.cu"
  [ -f "$f" ] || { models=0; break; }
  sed -n '/^__global__ void generate[A-Za-z]*Device(/,/^}/p' "$f" > "$here/_ref/model_$m.inc"
  grep -q '^}' "$here/_ref/model_$m.inc" || models=0
done
for m in circle_center circle_uniform_center; do
  f="$ref/source/nbfmm/model/$m.cu"
  [ -f "$f" ] || { models=0; break; }
  sed -n '/const float2 effect = kernelFunction(/,/const float angle_difference = /p' "$f" \
    > "$here/_ref/model_${m}_host.inc"
  [ "$(wc -l < "$here/_ref/model_${m}_host.inc")" -eq 2 ] || models=0
done
if [ "$models" = 1 ]; then defs="$defs -DNBFMM_REF_MODELS"; fi
${CXX:-g++} -O2 -ffp-contract=off -fPIC -shared $defs -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP \
  -I"$here/_ref" -I"$here/_ref/include" -I"$ref/include" -I"$cuda/include/cccl" -I"$cuda/include" \
  "$here/ref_shim.cpp" -o "$here/_ref/libnbfmm_refcpu.so"
echo "build_ref: wrote $here/_ref/libnbfmm_refcpu.so"
