#!/bin/sh
# Build oracle/_ref/refkern.cubin: the reference's own kernel source
# (TwoScale2D/WCSPHSolver.cu lines 14-2283: constants, device functions, kernels)
# compiled for sm_103a with the reference's compiler settings (nvcc defaults: -O3,
# contraction on, IEEE division and square root), between refgpu_shim.cuh and
# refgpu_entry.inc.  The source is streamed from the reference checkout into nvcc;
# nothing of it is written to disk.  The cubin is device code only, so it runs on
# any host: refgpu_launcher.cu loads it with the driver API.
# Usage: build_refgpu.sh REFERENCE_ROOT   (the directory holding the reference checkout)
set -e
[ -n "$1" ] || { echo "usage: $0 REFERENCE_ROOT (the reference checkout)" >&2; exit 2; }
REF=$1
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/../_ref"
CUR="$REF/TwoScale2D/WCSPHSolver.cu"
[ -f "$CUR" ] || { echo "reference source not found under $REF" >&2; exit 2; }
mkdir -p "$OUT"
NVCC=${NVCC:-nvcc}
{
  echo '#include "refgpu_shim.cuh"'
  echo "#line 14 \"$CUR\""
  sed -n '14,2283p' "$CUR"
  echo '#line 1 "refgpu_entry.inc"'
  echo '#include "refgpu_entry.inc"'
} | "$NVCC" -x cu -cubin -gencode arch=compute_103a,code=sm_103a -O3 -w -I"$HERE" -o "$OUT/refkern.cubin" -
echo "built $OUT/refkern.cubin"
