#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_build/.
# Same flags on x86_64 and aarch64: -ffp-contract=off keeps every rounding
# step explicit so both machines produce identical results.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
g++ -std=c++17 -O2 -fopenmp -ffp-contract=off -fPIC -shared \
    -o "$here/_build/libknnsj_oracle.so" "$here/knnsj_oracle.cpp"
