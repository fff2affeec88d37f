#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.
# Portable C only: no -march flags, no intrinsics, so the same source builds on
# x86_64 and aarch64 hosts.  No fast-math and no FMA contraction, so float
# rounding follows the C source operation by operation.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
${CC:-gcc} -O2 -std=c11 -fPIC -shared -fopenmp -fno-fast-math -ffp-contract=off \
  -o "$here/_build/liboracle.so.tmp" "$here/flowreg_oracle.c" -lm
mv -f "$here/_build/liboracle.so.tmp" "$here/_build/liboracle.so"
