"""Pins the FP64 oracle to the reference's own force functors.

The fixtures in tests/golden hold outputs of the reference's
CalcForceEpEpWithLinearCutoffNoSimd / CalcForceEpSpQuadNoSimd /
SearchNeighborEpEpNoSimd (src/soft_force.hpp) and of its AVX-512
PhantomGrapeQuad kernels (src/phantomquad_for_p3t_x86.hpp), compiled from the
reference sources by oracle/ref/build_ref.sh and run by
tests/golden/make_golden.py.
"""
import numpy as np
import pytest

import oracle
from helpers import load_golden, rel_err, rel_err_vec

CASES = ["kernel_test", "kernel_test_rsvar", "plummer2048_walks"]


@pytest.mark.parametrize("case", CASES)
def test_oracle_bit_exact_vs_reference_nosimd(case):
    """Same expressions, same order, no FMA contraction: bit-for-bit equal."""
    wb, d = load_golden(case)
    o = oracle.force(wb, nnb_with_eps=False, parts=True)
    np.testing.assert_array_equal(o["acc_ep"], d["nosimd__acc_ep"])
    np.testing.assert_array_equal(o["pot_ep"], d["nosimd__pot_ep"])
    np.testing.assert_array_equal(o["acc_sp"], d["nosimd__acc_sp"])
    np.testing.assert_array_equal(o["pot_sp"], d["nosimd__pot_sp"])
    np.testing.assert_array_equal(o["nnb"], d["nosimd__nnb_ep"])
    np.testing.assert_array_equal(o["nnb"], d["nosimd__nnb_search"])


@pytest.mark.parametrize("case", CASES)
def test_oracle_vs_reference_avx512_fp32(case):
    """PeTar's default CPU path: FP32 on absolute coordinates, EP rsqrt with one
    Newton step, SP raw rsqrt.  The reference's own kernel test bound is
    DF_MAX = 7e-3 (src/simd_test.cxx:68); the observed agreement is far tighter,
    and the neighbour counts agree exactly on these inputs."""
    wb, d = load_golden(case)
    o = oracle.force(wb, nnb_with_eps=False, parts=True)
    assert rel_err_vec(d["simd32__acc_ep"], o["acc_ep"]).max() < 1e-4
    assert rel_err(d["simd32__pot_ep"], o["pot_ep"]).max() < 1e-4
    assert rel_err_vec(d["simd32__acc_sp"], o["acc_sp"]).max() < 7e-3
    assert rel_err(d["simd32__pot_sp"], o["pot_sp"]).max() < 7e-3
    np.testing.assert_array_equal(o["nnb"], d["simd32__nnb_ep"])
    np.testing.assert_array_equal(o["nnb"], d["simd32__nnb_search"])


@pytest.mark.parametrize("case", CASES)
def test_oracle_vs_reference_avx512_fp64_forces(case):
    """PhantomGrapeQuad64Bit forces agree to FP64 rounding.  Its AVX-512
    neighbour count compares r^2 with max(rs_i, rs_j) instead of its square
    (src/phantomquad_for_p3t_x86.hpp:1705,1827), so those counts are not a
    parity reference; the test records that they disagree."""
    wb, d = load_golden(case)
    o = oracle.force(wb, nnb_with_eps=False, parts=True)
    assert rel_err_vec(d["simd64__acc_ep"], o["acc_ep"]).max() < 1e-12
    assert rel_err(d["simd64__pot_ep"], o["pot_ep"]).max() < 1e-12
    assert rel_err_vec(d["simd64__acc_sp"], o["acc_sp"]).max() < 1e-12
    assert rel_err(d["simd64__pot_sp"], o["pot_sp"]).max() < 1e-12
    assert (d["simd64__nnb_ep"] >= o["nnb"]).all()
    assert (d["simd64__nnb_ep"] != o["nnb"]).any()


def test_gpu_neighbour_semantics_include_eps2():
    """The GPU functor tests r2 + eps2 (src/force_gpu_cuda.cu:62-64), NoSimd
    tests r2 (src/soft_force.hpp:62): with eps > 0 the GPU form counts fewer or
    equal, and with eps = 0 both agree."""
    wb, _ = load_golden("kernel_test")
    gpu_sem = oracle.force(wb, nnb_with_eps=True)["nnb"]
    nosimd_sem = oracle.force(wb, nnb_with_eps=False)["nnb"]
    assert (gpu_sem <= nosimd_sem).all()
    wb.eps2 = 0.0
    np.testing.assert_array_equal(oracle.force(wb, nnb_with_eps=True)["nnb"],
                                  oracle.force(wb, nnb_with_eps=False)["nnb"])


def test_oracle_total_is_sum_of_parts():
    wb, _ = load_golden("plummer2048_walks")
    o = oracle.force(wb, parts=True)
    np.testing.assert_array_equal(o["acc"], (0.0 + o["acc_ep"]) + o["acc_sp"])
    np.testing.assert_array_equal(o["pot"], (0.0 + o["pot_ep"]) + o["pot_sp"])
