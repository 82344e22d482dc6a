#!/bin/sh
# Compiles the reference MaBoSSG's three device-kernel files, unmodified and where they lie in a
# reference checkout, to the LTO fatbins its JIT links against (the reference's own build makes the
# same files with `-arch lto_<cc> -rdc=true -fatbin`; cc = 103 on a GB300). Baseline measurement
# only. Usage: sh baseline/refgpu/build_kernels.sh <reference checkout>   (writes baseline/_ref/)
set -e
REF="$1"
if [ -z "$REF" ] || [ ! -f "$REF/src/jit_kernels/simulation.cu" ]; then
  echo "usage: sh baseline/refgpu/build_kernels.sh <reference checkout holding src/jit_kernels/>" >&2
  exit 2
fi
OUT="$(dirname "$0")/../_ref"
mkdir -p "$OUT"
NVCC="${CUDA_HOME:-/usr/local/cuda}/bin/nvcc"
for k in simulation final_states window_average_small; do
  "$NVCC" -arch=lto_103 -rdc=true -fatbin -o "$OUT/$k.fatbin" "$REF/src/jit_kernels/$k.cu"
done
ls -l "$OUT"
