#!/bin/sh
# Build oracle/_ref/librefcpu.so: the reference's own kernel source
# (TwoScale2D/WCSPHSolver.cu, lines 14-2283: constants, device functions and
# __global__ kernels, in namespace `cur`; plus TwoScale2D-master/TwoScale2D/WCSPHSolver.cu lines
# 14-1747 in namespace `older`, for the relaxation kernels) compiled for the CPU
# with cuda_shim.h and driven by refcpu_harness.inc.  The source is streamed from
# the reference checkout into the compiler; nothing of it is written to disk.
# Usage: build_ref.sh REFERENCE_ROOT   (the directory holding the reference checkout)
set -e
[ -n "$1" ] || { echo "usage: $0 REFERENCE_ROOT (the reference checkout)" >&2; exit 2; }
REF=$1
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/../_ref"
CUR="$REF/TwoScale2D/WCSPHSolver.cu"
OLD="$REF/TwoScale2D-master/TwoScale2D/WCSPHSolver.cu"
[ -f "$CUR" ] && [ -f "$OLD" ] || { echo "reference sources not found under $REF" >&2; exit 2; }
mkdir -p "$OUT"
{
  echo '#include "cuda_shim.h"'
  echo 'namespace cur {'
  echo "#line 14 \"$CUR\""
  sed -n '14,2283p' "$CUR"
  echo '}'
  echo 'namespace older {'
  echo "#line 14 \"$OLD\""
  sed -n '14,1747p' "$OLD"
  echo '}'
  echo '#line 1 "refcpu_harness.inc"'
  echo '#include "refcpu_harness.inc"'
} | g++ -x c++ -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -w \
      -I"$HERE" -I"$HERE/../../include" -o "$OUT/librefcpu.so" -
echo "built $OUT/librefcpu.so"
