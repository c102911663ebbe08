#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_build/.
# vefem_stability_oracle.c includes vefem_oracle.c: one library with both;
# libvefem_oracle_cs.so is vefem_oracle.c built on complex numbers.
# -ffp-contract=off: no FMA contraction, plain IEEE binary64 in source order.
# -O3 for the timed CPU baseline; no -march=native: the same source is built on
# x86-64 here and on the aarch64 GPU host, and must give the same bits on both
# (with contraction off, vector code would not change any result anyway).
# The flags are written next to the library so the benchmark can report them.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$HERE/_build"
OMP="-fopenmp"
if ! echo 'int main(void){return 0;}' | gcc -x c -fopenmp - -o /dev/null 2>/dev/null; then OMP=""; fi
FLAGS="-O3 -std=c11 -ffp-contract=off -fno-fast-math -fPIC -shared $OMP"
gcc $FLAGS -o "$HERE/_build/libvefem_oracle.so.tmp" "$HERE/vefem_stability_oracle.c" -lm
mv "$HERE/_build/libvefem_oracle.so.tmp" "$HERE/_build/libvefem_oracle.so"
# the same routines on complex numbers: the complex-step exact Jacobian
gcc $FLAGS -DORA_COMPLEX_STEP -o "$HERE/_build/libvefem_oracle_cs.so.tmp" "$HERE/vefem_oracle.c" -lm
mv "$HERE/_build/libvefem_oracle_cs.so.tmp" "$HERE/_build/libvefem_oracle_cs.so"
echo "gcc $(gcc -dumpfullversion) $FLAGS" > "$HERE/_build/flags.txt"
