#!/bin/sh
# Builds the CPU oracle (test infrastructure only) into oracle/_build/.
# -ffp-contract=off: no fused multiply-add, so the REF22 increments follow
# the plain (a*b + c*d) + e*f rounding on every host.
set -e
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
${CC:-gcc} -O2 -fPIC -shared -fopenmp -ffp-contract=off -std=gnu11 \
    -o "$here/_build/liboracle.so" "$here/discus_oracle.c" -lm
# The same source with the reference's release flags (its Fortran flags
# -O3 -ffast-math, with OpenMP): used only to time the reference's loops.
${CC:-gcc} -O3 -ffast-math -fPIC -shared -fopenmp -std=gnu11 \
    -o "$here/_build/liboracle_timing.so" "$here/discus_oracle.c" -lm
