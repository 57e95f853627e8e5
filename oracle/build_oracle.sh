#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure): oracle/_build/libnn_exact.so
# Portable flags only (the same recipe runs on x86_64 and aarch64 hosts).
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
gcc -O2 -fPIC -shared -fopenmp -std=c11 -o "$here/_build/libnn_exact.so.tmp" "$here/nn_exact.c" -lm
mv -f "$here/_build/libnn_exact.so.tmp" "$here/_build/libnn_exact.so"
