#!/usr/bin/env bash
# Builds oracle/_ref/libi2ref.so from the reference's own sources (andreyypopov/integrator2,
# src/) compiled for the HOST through oracle/ref_shim.h, plus oracle/ref_driver.cu.
# TEST INFRASTRUCTURE ONLY: used to generate and re-check tests/golden/.  Needs the reference
# checkout (default /root/reference, override with I2_REFERENCE); skipped when it is absent.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${I2_REFERENCE:-/root/reference}"
out="$here/_ref"
if [ ! -d "$ref/src" ]; then
    echo "ref_build: no reference sources at $ref; skipped" >&2
    exit 0
fi
mkdir -p "$out"
# where the checkout was found, for tests that compile the reference's own test program
(cd "$ref" && pwd) > "$out/reference_path"
flags=(-x cu -std=c++17 -O2 -rdc=true -Xcompiler -fPIC -Xcompiler -ffp-contract=off
       -Xcompiler -Wno-deprecated-declarations -diag-suppress 1444,20091,20092
       -include "$here/ref_shim.h" -I"$ref/src"
       -gencode arch=compute_103a,code=sm_103a)
srcs=(evaluators/evaluatorJ3DK.cu evaluators/evaluator3d.cu NumericalIntegrator3d.cu Mesh3d.cu
      common/cuda_math.cu common/cuda_helper.cu)
objs=()
pids=()
for s in "${srcs[@]}"; do
    o="$out/$(basename "$s" .cu).o"
    nvcc "${flags[@]}" -c "$ref/src/$s" -o "$o" &
    pids+=($!)
    objs+=("$o")
done
nvcc "${flags[@]}" -c "$here/ref_driver.cu" -o "$out/ref_driver.o" &
pids+=($!)
objs+=("$out/ref_driver.o")
for p in "${pids[@]}"; do wait "$p"; done
nvcc -shared -rdc=true -gencode arch=compute_103a,code=sm_103a -Xcompiler -fPIC "${objs[@]}" -o "$out/libi2ref.so"
rm -f "${objs[@]}"
echo "ref_build: $out/libi2ref.so"
