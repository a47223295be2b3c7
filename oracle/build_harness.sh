#!/bin/sh
# Builds the headless reference runner oracle/_build/libref_harness.so
# (test infrastructure; links the CUDA driver library).
set -e
here=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$here/_build"
CUDA=${CUDA_HOME:-/usr/local/cuda}
${CXX:-g++} -O2 -std=c++17 -fPIC -shared -I"$CUDA/include" \
  "$here/ref_harness.cpp" -o "$here/_build/libref_harness.so" \
  -L"$CUDA/lib64/stubs" -L"$CUDA/lib64" -lcuda
