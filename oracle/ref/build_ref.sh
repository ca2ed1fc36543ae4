#!/usr/bin/env bash
# Compiles the reference's own CPU force functors from the reference sources,
# in place, into oracle/_ref/ (git-ignored):
#   libref_nosimd.so   FP64 NoSimd functors          (src/soft_force.hpp)
#   libref_simd32.so   AVX-512 PhantomGrapeQuad FP32  (src/phantomquad_for_p3t_x86.hpp),
#                      EP with one Newton-Raphson step as PeTar's default
#                      (RSQRT_NR_EPJ_X2, src/petar.hpp:1-15)
#   libref_simd64.so   AVX-512 PhantomGrapeQuad64Bit  (P3T_64BIT: CALC_EP_64bit,
#                      CALC_SP_64bit, RSQRT_NR_EPJ_X4, RSQRT_NR_SPJ_X4)
#   libref_changeover.so  changeover W functions      (src/changeover.hpp; SDAR's
#                      Common/Float.h replaced by oracle/ref/shim/Common/Float.h)
#   libref_kdkdk.so    NoSimd functors built with KDKDK_4TH, for the gradient
#                      correction CalcCorrectEpEpWithLinearCutoffNoSimd
# The SIMD kernels are x86 only; on other hosts only the NoSimd library is
# built.  The NoSimd build uses -ffp-contract=off so its FP64 results are
# defined by source order alone.
# Usage: oracle/ref/build_ref.sh REFERENCE_ROOT   (or PETAR_REFERENCE_ROOT in the environment)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${PETAR_REFERENCE_ROOT:-}}"
if [ -z "$REF" ]; then
    echo "usage: $0 REFERENCE_ROOT (the PeTar checkout whose src/ holds soft_force.hpp)" >&2
    exit 2
fi
SRC="$REF/src"
OUT="$HERE/../_ref"
if [ ! -f "$SRC/soft_force.hpp" ]; then
    echo "reference sources not found under $SRC" >&2
    exit 1
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
COMMON=(-std=c++17 -fPIC -shared -fopenmp -I"$HERE" -I"$SRC" -DUSE_QUAD)
"$CXX" -O2 -ffp-contract=off "${COMMON[@]}" -DREF_NOSIMD "$HERE/ref_driver.cpp" -o "$OUT/libref_nosimd.so" &
if [ "$(uname -m)" = "x86_64" ]; then
    SIMD=(-O2 -march=skylake-avx512 -DUSE_SIMD -DINTRINSIC_X86)
    "$CXX" "${SIMD[@]}" "${COMMON[@]}" -DREF_SIMD -DRSQRT_NR_EPJ_X2 \
        "$HERE/ref_driver.cpp" -o "$OUT/libref_simd32.so" &
    "$CXX" "${SIMD[@]}" "${COMMON[@]}" -DREF_SIMD -DCALC_EP_64bit -DCALC_SP_64bit \
        -DRSQRT_NR_EPJ_X4 -DRSQRT_NR_SPJ_X4 "$HERE/ref_driver.cpp" -o "$OUT/libref_simd64.so" &
fi
"$CXX" -O2 -ffp-contract=off "${COMMON[@]}" -DREF_NOSIMD -DKDKDK_4TH "$HERE/ref_driver.cpp" \
    -o "$OUT/libref_kdkdk.so" &
"$CXX" -O2 -ffp-contract=off -std=c++17 -fPIC -shared -I"$HERE/shim" -I"$SRC" \
    "$HERE/ref_changeover.cpp" -o "$OUT/libref_changeover.so" &
wait
ls "$OUT"
