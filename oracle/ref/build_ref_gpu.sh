#!/usr/bin/env bash
# Compiles the device code of the reference's CUDA soft-force file
# (src/force_gpu_cuda.cu: force_kernel_ep_ep, force_kernel_ep_sp and the
# device functions they call) for sm_103a into oracle/_ref/ref_force_gpu.cubin
# (git-ignored), as PeTar's default GPU build configures it
# (PARTICLE_SIMULATOR_GPU_MULIT_WALK_INDEX, USE_QUAD, GPU_PROFILE).
#
# The file is read where it lies and piped to nvcc with its two FDPS/PeTar
# includes (<particle_simulator.hpp>, "force_gpu_cuda.hpp", which pull in the
# whole of FDPS and PeTar) replaced by oracle/ref/gpushim/pgf_ref_gpu_shim.hpp;
# nothing of it is written to disk.  The cubin holds GPU code only, so
# oracle/ref/ref_gpu_driver.cu loads it on any host with the driver API.
# Usage: oracle/ref/build_ref_gpu.sh REFERENCE_ROOT   (or PETAR_REFERENCE_ROOT)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${PETAR_REFERENCE_ROOT:-}}"
if [ -z "$REF" ]; then
    echo "usage: $0 REFERENCE_ROOT (the PeTar checkout whose src/ holds force_gpu_cuda.cu)" >&2
    exit 2
fi
SRC="$REF/src"
OUT="$HERE/../_ref"
if [ ! -f "$SRC/force_gpu_cuda.cu" ]; then
    echo "reference sources not found under $SRC" >&2
    exit 1
fi
mkdir -p "$OUT"
NVCC="${NVCC:-nvcc}"
sed -e 's|^#include *<particle_simulator.hpp>|#include "pgf_ref_gpu_shim.hpp"|' \
    -e 's|^#include *"force_gpu_cuda.hpp"||' "$SRC/force_gpu_cuda.cu" |
    "$NVCC" -gencode arch=compute_103a,code=sm_103a -O3 -cubin -x cu -I"$HERE/gpushim" -I"$SRC" \
        -DPARTICLE_SIMULATOR_GPU_MULIT_WALK_INDEX -DUSE_QUAD -DGPU_PROFILE -o "$OUT/ref_force_gpu.cubin.tmp" -
mv "$OUT/ref_force_gpu.cubin.tmp" "$OUT/ref_force_gpu.cubin"
