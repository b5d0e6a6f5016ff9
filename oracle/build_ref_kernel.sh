#!/usr/bin/env bash
# Compiles the reference's own range-search kernel file (kernel.cu, with its
# headers) from its sources where they lie into a device-code-only cubin
# for one (DTYPE, GPUNUMDIM, NUMINDEXEDDIM) configuration:
# oracle/_ref/refkernel_<dtype>_<ndim>_<nidx>.cubin.
#
# TEST INFRASTRUCTURE ONLY.  The cubin holds the reference's
# kernelNDGridIndexGlobalkNN (kernel.cu:61-113 with evaluateCell/evalPoint);
# oracle/ref_kernel_runner.cpp loads it with the CUDA driver API on the GPU
# box so that tests can run the reference kernel itself against the CPU
# oracle.  A cubin is device code only, so the one built here runs on the
# Arm GPU machine as well.
#
# As in build_ref_host.sh, a scratch directory of symlinks points at the
# reference files and holds a params.h written with the reference's own sed
# edits (Makefile:70-71); -std=c++17 because CUDA 13's CCCL rejects C++14.
#
# usage: build_ref_kernel.sh <float|double> <GPUNUMDIM> <NUMINDEXEDDIM> [REFDIR]
set -euo pipefail
dtype="$1"; ndim="$2"; nidx="$3"
refdir="${4:-/root/reference}"
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
out="$here/_ref/refkernel_${dtype}_${ndim}_${nidx}.cubin"
mkdir -p "$here/_ref"
work="$(mktemp -d /tmp/knnsj_refkern.XXXXXX)"
trap 'rm -rf "$work"' EXIT
for f in kernel.cu kernel.h kernelloops.h structs.h; do
  ln -s "$refdir/$f" "$work/$f"
done
sed -e "s/#define GPUNUMDIM.*/#define GPUNUMDIM $ndim/" \
    -e "s/#define NUMINDEXEDDIM.*/#define NUMINDEXEDDIM $nidx/" \
    -e "s/#define DTYPE.*/#define DTYPE $dtype/" \
    "$refdir/params.h" > "$work/params.h"
(cd "$work" && nvcc -std=c++17 -O3 -w -cubin -gencode arch=compute_103a,code=sm_103a kernel.cu -o "$out")
