#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_build/:
#  liboracle.so          the checker: portable C, -O2, no -march flags, no
#                        fast-math and no FMA contraction, so float rounding
#                        follows the C source operation by operation and the
#                        same source gives the same bits on x86_64 and aarch64;
#  liboracle_o3.so       the timed CPU baseline: the same source and the same
#                        float semantics (no contraction, no fast-math), built
#                        with -O3 (portable: no -march flags either), so it
#                        returns the checker's bits, only faster;
#  liboracle_fastmath.so the same with -ffast-math, the analogue of the
#                        reference's numba @njit(fastmath=True): timed only,
#                        its flows differ from the checker's in rounding.
# The flags used are written to _build/flags.txt.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
cc=${CC:-gcc}
src="$here/flowreg_oracle.c"
base="-std=c11 -fPIC -shared -fopenmp"
$cc -O2 $base -fno-fast-math -ffp-contract=off -o "$here/_build/liboracle.so.tmp" "$src" -lm
mv -f "$here/_build/liboracle.so.tmp" "$here/_build/liboracle.so"
nflags="-O3 -fno-fast-math -ffp-contract=off"
fflags="-O3 -ffast-math"
$cc $nflags $base -o "$here/_build/liboracle_o3.so.tmp" "$src" -lm
mv -f "$here/_build/liboracle_o3.so.tmp" "$here/_build/liboracle_o3.so"
$cc $fflags $base -o "$here/_build/liboracle_fastmath.so.tmp" "$src" -lm
mv -f "$here/_build/liboracle_fastmath.so.tmp" "$here/_build/liboracle_fastmath.so"
printf 'o3: %s %s\nfastmath: %s %s\n' "$cc" "$nflags" "$cc" "$fflags" > "$here/_build/flags.txt"
