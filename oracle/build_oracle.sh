#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_build/.
# Same flags on x86_64 and aarch64: -ffp-contract=off keeps every rounding
# step explicit so both machines produce identical results.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
g++ -std=c++17 -O2 -fopenmp -ffp-contract=off -fPIC -shared \
    -o "$here/_build/libknnsj_oracle.so" "$here/knnsj_oracle.cpp"
# runner of the reference's range-search kernel from a cubin (CUDA driver API)
cuda="${CUDA_HOME:-/usr/local/cuda}"
g++ -std=c++17 -O2 -fPIC -shared -I"$cuda/include" \
    -o "$here/_build/libref_kernel_runner.so" "$here/ref_kernel_runner.cpp" \
    -L"$cuda/lib64/stubs" -L"$cuda/lib64" -lcuda
