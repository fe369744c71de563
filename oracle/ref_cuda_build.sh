#!/usr/bin/env bash
# Builds oracle/_ref/ref_kernels.cubin: the reference's own CUDA sources (andreyypopov/integrator2,
# src/, unmodified, through oracle/ref_unit.cu) compiled for sm_103a, plus
# oracle/_ref/ref_kernels.names, the mangled names of its kernels (read with nm from a host
# object of the same unit).  TEST INFRASTRUCTURE ONLY: oracle/ref_cuda.py launches these kernels
# on the GPU machine to check the library against the reference's own CUDA build and to time it.
# Needs the reference checkout (default /root/reference, override with I2_REFERENCE); skipped
# when it is absent (the GPU machine uses the files built here).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${I2_REFERENCE:-/root/reference}"
out="$here/_ref"
if [ ! -d "$ref/src" ]; then
    echo "ref_cuda_build: no reference sources at $ref; skipped" >&2
    exit 0
fi
mkdir -p "$out"
flags=(-std=c++17 -O3 -I"$ref/src" -diag-suppress 1444,20091,20092 -Xcompiler -Wno-deprecated-declarations)
nvcc -gencode arch=compute_103a,code=sm_103a "${flags[@]}" -cubin "$here/ref_unit.cu" -o "$out/ref_kernels.cubin" &
p1=$!
nvcc -gencode arch=compute_103a,code=sm_103a "${flags[@]}" -c "$here/ref_unit.cu" -o "$out/ref_unit_host.o" &
p2=$!
wait $p1
wait $p2
nm -g --defined-only "$out/ref_unit_host.o" | awk '$2 == "T" && $3 ~ /^_Z[0-9]+k[A-Z]/ {print $3}' > "$out/ref_kernels.names"
rm -f "$out/ref_unit_host.o"
echo "ref_cuda_build: $out/ref_kernels.cubin ($(wc -l < "$out/ref_kernels.names") kernels)"
