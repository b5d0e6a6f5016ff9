#!/usr/bin/env bash
# Builds the reference's own host code from its sources where they lie, for
# one (DTYPE, GPUNUMDIM, NUMINDEXEDDIM) configuration, and links it with
# oracle/ref_host_driver.cpp into oracle/_ref/ref_host_<tag>.
#
# TEST INFRASTRUCTURE ONLY (fixture generation, run in the build container
# where the reference is mounted; nothing here runs on a GPU).
#
# The reference sets its knobs in params.h and its own Python build rewrites
# that file in place with sed (Makefile:70-71).  The reference tree is
# read-only, so this recipe points a scratch directory of symlinks at the
# reference files and writes the per-configuration params.h there with the
# same sed edits.  Compile flags follow Makefile:16 with -std=c++17 (CUDA 13's
# CCCL rejects C++14) and `-include thrust/unique.h` for GPU.cu (GPU.cu:3886
# calls thrust::unique without including it).  Objects and the driver go to
# oracle/_ref/ only.
#
# usage: build_ref_host.sh <float|double> <GPUNUMDIM> <NUMINDEXEDDIM> [REFDIR]
set -euo pipefail
dtype="$1"; ndim="$2"; nidx="$3"
refdir="${4:-/root/reference}"
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
tag="${dtype}_${ndim}_${nidx}"
out="$here/_ref/$tag"
mkdir -p "$out"
work="$(mktemp -d /tmp/knnsj_refsrc.XXXXXX)"
trap 'rm -rf "$work"' EXIT
for f in main.cu GPU.cu GPU.h kernel.cu kernel.h kernelloops.h structs.h \
         import_dataset.cpp par_sort.cpp par_sort.h; do
  ln -s "$refdir/$f" "$work/$f"
done
sed -e "s/#define GPUNUMDIM.*/#define GPUNUMDIM $ndim/" \
    -e "s/#define NUMINDEXEDDIM.*/#define NUMINDEXEDDIM $nidx/" \
    -e "s/#define DTYPE.*/#define DTYPE $dtype/" \
    "$refdir/params.h" > "$work/params.h"
arch="-gencode arch=compute_100,code=sm_100"
flags="-std=c++17 -O3 -Xcompiler -fopenmp -Xcompiler -fPIC -DPYTHON -w"
(cd "$work" && g++ -O3 -fPIC -c par_sort.cpp -o "$out/par_sort.o") &
(cd "$work" && nvcc $flags $arch -c import_dataset.cpp -o "$out/import_dataset.o") &
(cd "$work" && nvcc $flags $arch -c kernel.cu -o "$out/kernel.o") &
(cd "$work" && nvcc $flags $arch -include thrust/unique.h -c GPU.cu -o "$out/GPU.o") &
(cd "$work" && nvcc $flags $arch -c main.cu -o "$out/main.o") &
wait
nvcc -std=c++17 -O2 -Xcompiler -fopenmp -DREF_DTYPE="$dtype" -DNUMINDEXEDDIM_BUILD="$nidx" \
    -o "$out/ref_host_driver" "$here/ref_host_driver.cpp" \
    "$out/main.o" "$out/GPU.o" "$out/kernel.o" "$out/import_dataset.o" "$out/par_sort.o" -lgomp
echo "$out/ref_host_driver"
