#!/usr/bin/env bash
# Builds the CPU oracle (test infrastructure) into oracle/_build/.
# vefem_stability_oracle.c includes vefem_oracle.c: one library with both.
# -ffp-contract=off: no FMA contraction, plain IEEE binary64 in source order.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$HERE/_build"
OMP="-fopenmp"
if ! echo 'int main(void){return 0;}' | gcc -x c -fopenmp - -o /dev/null 2>/dev/null; then OMP=""; fi
gcc -O2 -std=c11 -ffp-contract=off -fno-fast-math -fPIC -shared $OMP \
    -o "$HERE/_build/libvefem_oracle.so.tmp" "$HERE/vefem_stability_oracle.c" -lm
mv "$HERE/_build/libvefem_oracle.so.tmp" "$HERE/_build/libvefem_oracle.so"
