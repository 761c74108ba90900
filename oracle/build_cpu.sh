#!/usr/bin/env bash
# Builds oracle/libgspec_cpu.so, the OpenMP C restatement of the chain used as
# the CPU baseline and as a second checker.  Portable flags only (the same
# recipe runs on x86-64 and aarch64).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
CC="${CC:-gcc}"
"$CC" -O3 -std=c11 -fopenmp -fPIC -shared -o "$HERE/libgspec_cpu.so" "$HERE/gspec_cpu.c" -lm
