#!/bin/sh
# Builds the reference-side checkers from the reference checkout, in place
# (default /root/reference; set BSF_REFERENCE_DIR to override):
#   oracle/_ref/libref_harness.so  the reference's host C++ headers (p20_exact_math.hpp,
#                                  coarse_exact_core.hpp, p19_monster_gate.hpp) behind
#                                  oracle/ref_harness.cpp, for golden vectors and CPU pins;
#   oracle/_ref/ref_worker.cubin   the device code of the reference worker
#                                  (native/src/gpu_p20_benchmark.cpp, unmodified) for
#                                  sm_103a with the reference's own nvcc flags
#                                  (native/CMakeLists.txt: -O3 --fmad=false --ftz=false
#                                  --prec-div=true --prec-sqrt=true), driven on the GPU by
#                                  oracle/ref_gpu.cpp.
# Test and bench infrastructure only; exits 0 without building when the checkout is absent.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${BSF_REFERENCE_DIR:-/root/reference}
if [ ! -f "$REF/native/src/p20_exact_math.hpp" ]; then
    echo "reference checkout not found at $REF; skipping oracle/_ref" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -I"$REF/native/src" \
    -o "$HERE/_ref/libref_harness.so" "$HERE/ref_harness.cpp"
echo "built $HERE/_ref/libref_harness.so"
CUBIN="$HERE/_ref/ref_worker.cubin"
NVCC=${NVCC:-nvcc}
if [ -f "$CUBIN" ] && [ -z "$(find "$REF/native/src" -newer "$CUBIN" -type f)" ]; then
    echo "up to date: $CUBIN"
    exit 0
fi
if command -v "$NVCC" >/dev/null 2>&1; then
    "$NVCC" -gencode arch=compute_103a,code=sm_103a -cubin -x cu -std=c++17 -O3 \
        --fmad=false --ftz=false --prec-div=true --prec-sqrt=true -DBSF_NVIDIA_CUDA=1 \
        -I"$REF/native/src" -w -o "$CUBIN.tmp" "$REF/native/src/gpu_p20_benchmark.cpp"
    mv "$CUBIN.tmp" "$CUBIN"
    echo "built $CUBIN"
fi
