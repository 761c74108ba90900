#!/usr/bin/env bash
# Builds oracle/_ref/libref_host.so from the reference's own sources where
# they lie (the psrdada_cpp tree given as the first argument or in
# PSRDADA_CPP_TREE; without either it builds nothing), with the stub headers
# in oracle/ref_shim/ standing in for googletest, Boost.Log and psrdada.
# The library exports the reference's host-side C reference functions
# (see oracle/ref_shim/ref_exports.cu); it is used only to pin the oracle.
# oracle/_ref/ref_kernels.cubin holds the reference's GPU kernels
# (oracle/ref_shim/ref_kernels.cu) for the GPU pin test.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${PSRDADA_CPP_TREE:-}}"
OUT="$HERE/_ref"
NVCC="${NVCC:-/usr/local/cuda/bin/nvcc}"
if [ -z "$REF" ]; then echo "no psrdada_cpp tree given (argument or PSRDADA_CPP_TREE): reference pin not built"; exit 0; fi
[ -d "$REF/psrdada_cpp" ] || { echo "reference tree not found at $REF" >&2; exit 2; }
mkdir -p "$OUT"
EDD="$REF/psrdada_cpp/effelsberg/edd"
FLAGS=(-std=c++17 -O2 -Xcompiler -fPIC -DENABLE_CUDA=1 -gencode arch=compute_103a,code=sm_103a
       -I "$HERE/ref_shim" -I "$REF" -w)
SRCS=("$EDD/test/src/UnpackerTester.cu" "$EDD/test/src/DetectorAccumulatorTester.cu"
      "$EDD/src/Unpacker.cu" "$EDD/src/GatedSpectrometer.cu" "$REF/psrdada_cpp/src/raw_bytes.cpp"
      "$HERE/ref_shim/ref_exports.cu" "$HERE/ref_shim/unused_symbols.cu")
OBJS=()
pids=()
for s in "${SRCS[@]}"; do
  b="$(basename "$s")"; o="$OUT/${b%.*}.o"
  OBJS+=("$o")
  "$NVCC" "${FLAGS[@]}" -x cu -c "$s" -o "$o" &
  pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
"$NVCC" -gencode arch=compute_103a,code=sm_103a -shared -o "$OUT/libref_host.so" "${OBJS[@]}" -lcudart
echo "built $OUT/libref_host.so"
# the reference's GPU kernels as one module for the driver API (the GPU pin
# test), with the kernels' symbol names as ptxas lists them
"$NVCC" "${FLAGS[@]}" -Xptxas -v -cubin -x cu "$HERE/ref_shim/ref_kernels.cu" -o "$OUT/ref_kernels.cubin" \
    2> "$OUT/ref_kernels.ptxas.txt"
sed -n "s/.*Compiling entry function '\([^']*\)'.*/\1/p" "$OUT/ref_kernels.ptxas.txt" | sort -u > "$OUT/ref_kernels.names"
echo "built $OUT/ref_kernels.cubin ($(wc -l < "$OUT/ref_kernels.names") kernels)"
