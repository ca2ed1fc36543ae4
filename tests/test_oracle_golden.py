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
from helpers import GOLDEN, load_golden, rel_err, rel_err_vec

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


def test_changeover_w_matches_reference():
    """The oracle's changeover W functions against the reference's ChangeOver
    (src/changeover.hpp) compiled from its source: bit-exact, single and pair
    forms, including the tie rule of the pair form."""
    d = dict(np.load(GOLDEN / "changeover_w.npz"))
    a, p = oracle.co_w(d["r_in"], d["r_out"], d["dr"])
    np.testing.assert_array_equal(a, d["acc0w"])
    np.testing.assert_array_equal(p, d["potw"])
    a2, p2 = oracle.co_w_two(d["r_in"], d["r_out"], d["r_in2"], d["r_out2"], d["dr"])
    np.testing.assert_array_equal(a2, d["acc0w_two"])
    np.testing.assert_array_equal(p2, d["potw_two"])


def test_changeover_mass_scaling_matches_reference():
    """make_changeover's radii follow ChangeOver::setR(m_fac, r_in, r_out)."""
    d = dict(np.load(GOLDEN / "changeover_w.npz"))
    scale = np.maximum(np.power(d["m_fac"], 1.0 / 3.0), 1.0)
    np.testing.assert_allclose(d["r_in"] * scale, d["r_in_mfac"], rtol=4e-16, atol=0)
    np.testing.assert_allclose(d["r_out"] * scale, d["r_out_mfac"], rtol=4e-16, atol=0)


def test_changeover_oracle_composition():
    """The oracle's correction sequence (linear-cutoff kernel, then the
    reference's per-neighbour correction) against the composite it must equal,
    evaluated directly: changeover force and potentials for neighbours,
    linear cutoff for everything else, self-potential removed."""
    from petar_gb300 import ics, walks
    cl = ics.make_plummer_cluster(9, 1500, 0.03, binary_fraction=0.3)
    wb, co = walks.make_changeover(walks.build_walks(cl), cl.r_in, cl.r_out, seed=3)
    o = oracle.force_changeover(wb, co)
    base = oracle.force(wb, parts=True)
    G, r_out2 = wb.G, wb.rcut2
    r_out = np.sqrt(r_out2)
    for w in range(wb.n_walk):
        for i in range(wb.epi_disp[w], wb.epi_disp[w + 1]):
            js = wb.id_epj[wb.epj_disp[w]:wb.epj_disp[w + 1]]
            dx = wb.epj_pos[js] - wb.epi_pos[i]
            r2 = (dx * dx).sum(1) + wb.eps2
            nb = (r2 < np.maximum(wb.epi_rs[i], wb.epj_rs[js]) ** 2) & (co.epj_id[js] != co.epi_id[i])
            m = wb.epj_mass[js]
            rmax = np.sqrt(np.maximum(r2, r_out2))
            r = np.sqrt(r2)
            pick_i = co.epi_r_out[i] > co.epj_r_out[js]
            rin = np.where(pick_i, co.epi_r_in[i], co.epj_r_in[js])
            rou = np.where(pick_i, co.epi_r_out[i], co.epj_r_out[js])
            wa, wp = oracle.co_w(rin, rou, np.where(nb, r, 1.0))
            single = (co.epj_status[js] == 0) & (co.epj_mass_backup[js] == 0)
            member = co.epj_status[js] < 0
            meff = np.where(single, m, np.where(member, co.epj_mass_backup[js], 0.0))
            rr = np.where(nb, r, 1.0)
            acc = np.where(nb[:, None], (m * (1 - wa) / rr ** 3)[:, None] * dx, (m / rmax ** 3)[:, None] * dx)
            pt = np.where(nb, -meff / rr, -m / rmax)
            ps = np.where(nb, -meff * (1 - wp) / rr, -m / rmax)
            self_pot = co.epi_self_mass[i] / r_out
            want_acc = G * acc.sum(0) + base["acc_sp"][i]
            want_pt = G * (pt.sum() + self_pot) + base["pot_sp"][i]
            want_ps = G * (ps.sum() + self_pot) + base["pot_sp"][i]
            scale = np.abs(G * acc).sum(0).max() + abs(base["acc_sp"][i]).max()
            assert np.abs(o["acc"][i] - want_acc).max() <= 1e-11 * scale
            assert abs(o["pot"][i] - want_pt) <= 1e-11 * (G * np.abs(pt).sum() + abs(base["pot_sp"][i]) + G * self_pot)
            assert abs(o["pot_soft"][i] - want_ps) <= 1e-11 * (G * np.abs(ps).sum() + abs(base["pot_sp"][i]) + G * self_pot)


def _gradient_batch(d):
    from petar_gb300.walks import WalkBatch
    return WalkBatch(epi_pos=d["epi_pos"], epi_rs=d["epi_rs"], epi_disp=d["epi_disp"], epj_pos=d["epj_pos"],
                     epj_mass=d["epj_mass"], epj_rs=d["epj_rs"], spj_pos=d["spj_pos"], spj_mass=d["spj_mass"],
                     spj_quad=d["spj_quad"], epj_disp=d["epj_disp"], id_epj=d["id_epj"], spj_disp=d["spj_disp"],
                     id_spj=d["id_spj"], eps2=float(d["eps"]) ** 2, rcut2=float(d["r_out"]) ** 2, G=float(d["G"]))


def test_gradient_correction_matches_reference():
    """The oracle's KDKDK_4TH gradient-correction pass against the reference's
    CalcCorrectEpEpWithLinearCutoffNoSimd and quadrupole EP-SP functors
    (compiled from source with KDKDK_4TH): bit-exact acorr, acc and pot."""
    d = dict(np.load(GOLDEN / "gradient_walks.npz"))
    o = oracle.gradient(_gradient_batch(d), d["epi_acc"], d["epj_acc"])
    np.testing.assert_array_equal(o["acorr"], d["ref__acorr"])
    np.testing.assert_array_equal(o["acc"], d["ref__acc"])
    np.testing.assert_array_equal(o["pot"], d["ref__pot"])


def test_rows_batch_equals_full_walks():
    """The single-row walks of tests.helpers.rows_batch (used to check a
    particle sample against the oracle) give bit-identical oracle results."""
    from helpers import rows_batch
    wb, _ = load_golden("plummer2048_walks")
    rows = np.array([0, 5, 100, 777, wb.epi_rs.size - 1])
    full = oracle.force(wb)
    part = oracle.force(rows_batch(wb, rows))
    for k in ("acc", "pot", "nnb"):
        np.testing.assert_array_equal(part[k], full[k][rows], err_msg=k)
