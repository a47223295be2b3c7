#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.
# -ffp-contract=off keeps the FP64 arithmetic identical on x86-64 and aarch64.
set -e
here=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$here/_build"
${CC:-gcc} -O3 -fopenmp -ffp-contract=off -fPIC -shared -std=c11 \
  -Wall -Wno-unused-function \
  "$here/yh_oracle.c" "$here/yh_oracle_tlm.c" -o "$here/_build/liboracle.so" -lm
