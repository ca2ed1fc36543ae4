"""Per-configuration parity on the GPU for the named benchmark configurations:

* Plummer 1,048,576 centres of mass with 50% binaries (theta 0.3,
  r_out 0.003), the bench workload: the default mixed-precision kernel and
  the plain FP64 kernel over all walks, checked against the FP64 oracle on
  the 20 most expensive walks, the 20 cheapest and 300 random ones.
* Plummer 65,536 (theta 0.3, r_out 0.008): the mixed kernel against the FP64
  oracle on all walks, and its error against FP64 direct N^2 summation, which
  must equal the tree's own error (the kernel adds nothing visible to it).
* King W0 = 7, N = 4,194,304, theta 0.4, r_out 0.0015: one force evaluation,
  checked against the oracle on a random sample of walks (the oracle on all
  4M i-particles would take minutes).
* 64 independent Plummer clusters, N log-uniform in [1024, 65536], 30%
  binaries, per-cluster r_out = 0.05 N^(-1/3), in one launch, against the
  oracle on all walks and against the plain FP64 kernel.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from helpers import MIXED_MAX, assert_mixed_parity, rel_err, rel_err_vec, stats
from petar_gb300 import gpuforce, ics, walks
from petar_gb300.gpuforce import PGF_PRECISION_FP64, PGF_PRECISION_MIXED

pytestmark = pytest.mark.gpu

MIXED_MEDIAN = 1e-6
MIXED_P999 = 1e-5


def _errors(res, o, rows=None):
    acc, pot, nnb = res["acc"], res["pot"], res["nnb"]
    if rows is not None:
        acc, pot, nnb = acc[rows], pot[rows], nnb[rows]
    np.testing.assert_array_equal(nnb, o["nnb"])
    return stats(rel_err_vec(acc, o["acc"])), stats(rel_err(pot, o["pot"]))


def test_plummer1m_bin50_headline_config():
    """The bench workload itself (1,572,864 particles, 10,882 walks): the
    default mixed-precision kernel at the full parity bar, the plain FP64
    kernel to 1e-12, counts exact for both; then the gradient pass."""
    cl = ics.make_plummer_cluster(3, 1048576, 0.003, binary_fraction=0.5, theta=0.3)
    wb = walks.build_walks(cl)
    assert cl.n == 1572864
    cost = wb.n_epi.astype(np.int64) * (wb.n_epj + 2 * wb.n_spj)
    by_cost = np.argsort(cost, kind="stable")
    by_cost = by_cost[wb.n_epi[by_cost] > 0]
    rng = np.random.default_rng(13)
    sw = np.unique(np.concatenate([by_cost[-20:], by_cost[:20], rng.choice(wb.n_walk, 300, replace=False)]))
    rows = np.concatenate([np.arange(wb.epi_disp[w], wb.epi_disp[w + 1]) for w in sw])
    o = oracle.force(wb.subset(sw))
    assert gpuforce.get_kernel_variant() == gpuforce.DEFAULT_KERNEL_VARIANT
    res = gpuforce.compute(wb, PGF_PRECISION_MIXED)
    assert_mixed_parity(res["acc"][rows], res["pot"][rows], res["nnb"][rows], o, label="C3 mixed")
    f64 = gpuforce.compute(wb, PGF_PRECISION_FP64)
    np.testing.assert_array_equal(f64["nnb"][rows], o["nnb"])
    assert rel_err_vec(f64["acc"][rows], o["acc"]).max() <= 1e-12
    assert rel_err(f64["pot"][rows], o["pot"]).max() <= 1e-12
    # Every particle: mixed against the FP64 kernel (the comparison bench.py gates on).
    np.testing.assert_array_equal(res["nnb"], f64["nnb"])
    for e in (rel_err_vec(res["acc"], f64["acc"]), rel_err(res["pot"], f64["pot"])):
        s = stats(e)
        assert s["median"] <= MIXED_MEDIAN and s["p999"] <= MIXED_P999 and s["max"] <= MIXED_MAX, s
    # The KDKDK_4TH gradient pass on the same walks, with the FP64 forces as
    # each particle's a_i: acorr, acc and pot at the full bar on the sample.
    acc = f64["acc"]
    gr = gpuforce.compute_gradient(wb, acc, acc)
    og = oracle.gradient(wb.subset(sw), acc[rows], acc)
    for key in ("acorr", "acc", "pot"):
        e = rel_err(gr[key][rows], og[key]) if key == "pot" else rel_err_vec(gr[key][rows], og[key])
        s = stats(e)
        assert s["median"] <= MIXED_MEDIAN and s["p999"] <= MIXED_P999 and s["max"] <= MIXED_MAX, (key, s)
    assert (gr["nnb"] == 0).all()


def test_plummer65k_against_oracle_and_direct_sum():
    cl = ics.make_plummer_cluster(2, 65536, 0.008)
    wb = walks.build_walks(cl)
    res = gpuforce.compute(wb, PGF_PRECISION_MIXED)
    o = oracle.force(wb)
    sa, sp = _errors(res, o)
    assert sa["median"] <= MIXED_MEDIAN and sa["p999"] <= MIXED_P999, sa
    assert sp["median"] <= MIXED_MEDIAN and sp["p999"] <= MIXED_P999, sp
    # Error against direct summation on 4096 targets: the tree's own error.
    rows = np.sort(np.random.default_rng(1).choice(wb.epi_rs.size, 4096, replace=False))
    acc_d, pot_d = oracle.direct(cl.pos, cl.mass, wb.epi_index[rows], wb.eps2, wb.rcut2)
    e_gpu = rel_err_vec(res["acc"][rows], acc_d)
    e_tree = rel_err_vec(o["acc"][rows], acc_d)
    # The kernel's own error (about 1e-7 against the oracle) shifts these
    # statistics by no more than the mixed-precision tolerances.
    assert np.median(e_tree) < 2e-3
    assert abs(np.median(e_gpu) - np.median(e_tree)) <= MIXED_MEDIAN
    assert abs(np.quantile(e_gpu, 0.999) - np.quantile(e_tree, 0.999)) <= MIXED_P999


def test_king4m_sampled_walks():
    cl = ics.make_king_cluster(7, 4194304, 0.0015, W0=7.0, theta=0.4)
    wb = walks.build_walks(cl)
    res = gpuforce.compute(wb, PGF_PRECISION_MIXED)
    sw = np.sort(np.random.default_rng(3).choice(wb.n_walk, 120, replace=False))
    rows = np.concatenate([np.arange(wb.epi_disp[w], wb.epi_disp[w + 1]) for w in sw])
    o = oracle.force(wb.subset(sw))
    sa, sp = _errors(res, o, rows)
    assert sa["median"] <= MIXED_MEDIAN and sa["p999"] <= MIXED_P999, sa
    assert sp["median"] <= MIXED_MEDIAN and sp["p999"] <= MIXED_P999, sp


def test_ensemble64_one_launch():
    rng = np.random.default_rng(5)
    ns = np.round(np.exp(rng.uniform(np.log(1024), np.log(65536), 64))).astype(int)
    bs = []
    for k, n in enumerate(ns):
        cl = ics.make_plummer_cluster(500 + k, int(n), 0.05 * n ** (-1 / 3), binary_fraction=0.3)
        b = walks.build_walks(cl)
        b.walk_rcut2 = np.full(b.n_walk, cl.r_out ** 2)
        bs.append(b)
    wb = walks.concat_batches(bs)
    res = gpuforce.compute(wb, PGF_PRECISION_MIXED)
    o = oracle.force(wb)
    sa, sp = _errors(res, o)
    assert sa["median"] <= MIXED_MEDIAN and sa["p999"] <= MIXED_P999, sa
    assert sp["median"] <= MIXED_MEDIAN and sp["p999"] <= MIXED_P999, sp
    f64 = gpuforce.compute(wb, PGF_PRECISION_FP64)
    np.testing.assert_array_equal(f64["nnb"], o["nnb"])
    assert rel_err_vec(f64["acc"], o["acc"]).max() <= 1e-12
