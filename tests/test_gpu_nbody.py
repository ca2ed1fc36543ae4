"""Device-resident tree step (pgf_nbody_*): the device list builder against
the host list builder, its forces against the dispatch path and the FP64
oracle, CUDA-graph runs against eager runs, and the 100-step kick-drift-kick
run of the King W0 = 7, N = 4,194,304 configuration (theta 0.4, r_out 0.0015,
dt = 1/1024) with per-step force errors on a random 4096-particle sample."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from helpers import rel_err, rel_err_vec, rows_batch, stats
from petar_gb300 import gpuforce, ics, nbody, walks
from petar_gb300.gpuforce import PGF_PRECISION_FP64, PGF_PRECISION_MIXED

pytestmark = pytest.mark.gpu

MIXED_MEDIAN = 1e-6
MIXED_P999 = 1e-5


def _clusters():
    yield "plummer2048", ics.make_plummer_cluster(1, 2048, 0.02, theta=0.3)
    yield "plummer20k_bin50", ics.make_plummer_cluster(21, 20000, 0.004, binary_fraction=0.5)
    yield "king30k", ics.make_king_cluster(3, 30000, 0.004, W0=7.0, theta=0.4)
    yield "plummer3000_theta0", ics.make_plummer_cluster(4, 3000, 0.02, theta=0.0)


@pytest.mark.parametrize("name", ["plummer2048", "plummer20k_bin50", "king30k", "plummer3000_theta0"])
def test_device_lists_equal_host_builder(name):
    cl = dict(_clusters())[name]
    host = walks.build_walks(cl)
    with nbody.DeviceNBody(cl) as h:
        dev = h.lists()
    np.testing.assert_array_equal(dev.epi_index, host.epi_index)
    for k in ("epi_disp", "epj_disp", "spj_disp", "id_epj", "id_spj"):
        np.testing.assert_array_equal(getattr(dev, k), getattr(host, k), err_msg=k)
    # Moments bit for bit (same arithmetic, no FMA contraction on either side).
    for k in ("spj_mass", "spj_pos", "spj_quad"):
        np.testing.assert_array_equal(getattr(dev, k), getattr(host, k), err_msg=k)


def _particle_order(res, wb):
    """Dispatch results (EPI rows) in particle order."""
    out = {k: np.empty_like(v) for k, v in res.items()}
    for k, v in res.items():
        out[k][wb.epi_index] = v
    return out


@pytest.mark.parametrize("precision", [PGF_PRECISION_MIXED, PGF_PRECISION_FP64])
def test_device_force_matches_dispatch_and_oracle(precision):
    cl = ics.make_plummer_cluster(21, 20000, 0.004, binary_fraction=0.5)
    wb = walks.build_walks(cl)
    with nbody.DeviceNBody(cl, precision=precision) as h:
        st = h.state()
        v = h.stats()["kernel_variant"]
    gpuforce.set_kernel_variant(v)
    gpuforce.set_walk_split(False)  # the device step runs every walk whole
    try:
        ref = _particle_order(gpuforce.compute(wb, precision), wb)
    finally:
        gpuforce.set_walk_split(True)
    np.testing.assert_array_equal(st["n_ngb"], ref["nnb"])
    # Same lists, same kernel: equal up to the host packing's rounding of
    # the quadrupoles, which the host compiler may contract differently.
    assert rel_err_vec(st["acc"], ref["acc"]).max() <= 1e-9
    assert rel_err(st["pot"], ref["pot"]).max() <= 1e-9
    o = _particle_order(oracle.force(wb), wb)
    np.testing.assert_array_equal(st["n_ngb"], o["nnb"])
    sa, sp = stats(rel_err_vec(st["acc"], o["acc"])), stats(rel_err(st["pot"], o["pot"]))
    tol = (MIXED_MEDIAN, MIXED_P999) if precision == PGF_PRECISION_MIXED else (1e-13, 1e-12)
    assert sa["median"] <= tol[0] and sa["p999"] <= tol[1], sa
    assert sp["median"] <= tol[0] and sp["p999"] <= tol[1], sp


def test_graph_run_equals_eager_run():
    cl = ics.make_king_cluster(5, 40000, 0.004, W0=7.0, theta=0.4)
    with nbody.DeviceNBody(cl) as a, nbody.DeviceNBody(cl) as b:
        a.run(6, 1.0 / 1024, graph=True)
        b.run(6, 1.0 / 1024, graph=False)
        sa, sb = a.state(), b.state()
        for k in ("pos", "vel", "acc", "pot", "n_ngb"):
            np.testing.assert_array_equal(sa[k], sb[k], err_msg=k)
        # The cached graph replays: 6 more steps each way stay equal.
        a.run(6, 1.0 / 1024, graph=True)
        b.run(6, 1.0 / 1024, graph=False)
        np.testing.assert_array_equal(a.state()["pos"], b.state()["pos"])
        assert a.stats()["steps"] == 12


def _sample_errors(h, rows_rng, k=4096):
    """Force errors of the last evaluation on k random particles against the
    FP64 oracle over the same lists, and the exact neighbour counts."""
    wb = h.lists()
    st = h.state()
    rows = np.sort(rows_rng.choice(h.n, k, replace=False))  # sorted-order rows
    o = oracle.force(rows_batch(wb, rows))
    idx = wb.epi_index[rows]
    np.testing.assert_array_equal(st["n_ngb"][idx], o["nnb"])
    return stats(rel_err_vec(st["acc"][idx], o["acc"])), stats(rel_err(st["pot"][idx], o["pot"]))


def test_king4m_kdk_100_steps_one_graph():
    """C4 as specified: 100 steps in one graph, the force error of a random
    4096-particle sample at every step (mixed precision against an FP64
    evaluation over the same lists, recorded inside the graph), that FP64
    evaluation pinned to the oracle at the first and the last step, and the
    energy change over the run."""
    cl = ics.make_king_cluster(7, 4194304, 0.0015, W0=7.0, theta=0.4)
    rng = np.random.default_rng(11)
    sample = np.sort(rng.choice(cl.n, 4096, replace=False))
    with nbody.DeviceNBody(cl) as h:
        h.set_sample(sample, 101)
        h.force()  # record 0: the initial forces

        def pin_fp64(rec):
            wb = h.lists()
            inv = np.empty(cl.n, np.int64)
            inv[wb.epi_index] = np.arange(cl.n)
            rows = inv[sample]
            o = oracle.force(rows_batch(wb, rows))
            np.testing.assert_array_equal(rec["n_ngb64"], o["nnb"])
            np.testing.assert_array_equal(rec["n_ngb"], o["nnb"])
            assert rel_err_vec(rec["acc64"], o["acc"]).max() <= 1e-12
            assert rel_err(rec["pot64"], o["pot"]).max() <= 1e-12

        pin_fp64(h.samples()[0])
        ek0, ep0 = h.energy()
        h.run(100, 1.0 / 1024, graph=True)
        assert h.stats()["steps"] == 100
        recs = h.samples()
        assert recs.shape == (101, 4096)
        pin_fp64(recs[100])
        for k in range(101):
            r = recs[k]
            np.testing.assert_array_equal(r["n_ngb"], r["n_ngb64"], err_msg=f"step {k}")
            sa = stats(rel_err_vec(r["acc"], r["acc64"]))
            sp = stats(rel_err(r["pot"], r["pot64"]))
            assert sa["median"] <= MIXED_MEDIAN and sa["p999"] <= MIXED_P999, (k, sa)
            assert sp["median"] <= MIXED_MEDIAN and sp["p999"] <= MIXED_P999, (k, sp)
        ek1, ep1 = h.energy()
        e0, e1 = ek0 + ep0, ek1 + ep1
        # Bound state, and the soft step alone keeps its energy to a small
        # fraction over 100 steps of 1/1024.
        assert e0 < 0 and abs((e1 - e0) / e0) < 1e-3, (e0, e1)


def test_energy_drift_mixed_equals_fp64():
    """The same 100-step run with the mixed and the plain FP64 kernels: the
    energy histories agree far below the drift the integrator itself makes."""
    cl = ics.make_king_cluster(9, 65536, 0.004, W0=7.0, theta=0.4)
    out = {}
    for prec in (PGF_PRECISION_MIXED, PGF_PRECISION_FP64):
        with nbody.DeviceNBody(cl, precision=prec) as h:
            e0 = sum(h.energy())
            h.run(100, 1.0 / 1024, graph=True)
            e1 = sum(h.energy())
            out[prec] = (e0, e1, h.state()["pos"])
    (m0, m1, mp), (d0, d1, dp) = out[PGF_PRECISION_MIXED], out[PGF_PRECISION_FP64]
    assert abs(m0 - d0) <= 1e-6 * abs(d0)
    drift_m, drift_d = (m1 - m0) / abs(m0), (d1 - d0) / abs(d0)
    assert abs(drift_m - drift_d) <= 1e-6, (drift_m, drift_d)
    assert np.abs(mp - dp).max() <= 1e-6 * np.abs(dp).max()


def test_list_overflow_is_reported_and_force_recovers():
    """Arrays sized exactly for the first build (capacity factor 1): a denser
    configuration overflows them inside a graph run, which reports
    PGF_ERR_CAPACITY without touching memory out of range; force() then grows
    the arrays, and the lists equal the host builder's again."""
    cl = ics.make_plummer_cluster(31, 20000, 0.004, binary_fraction=0.3)
    with nbody.DeviceNBody(cl, list_capacity_factor=1.0) as h:
        dense = cl.pos * 0.01  # r_search boxes now reach far more cells: EPJ lists double
        h.set_state(pos=dense)
        with pytest.raises(gpuforce.GpuForceError) as e:
            h.run(1, 1e-9, graph=True)
        assert e.value.code == 5, e.value
        h.set_state(pos=dense, vel=cl.vel)
        h.force()
        dev = h.lists()
    cl.pos = dense
    host = walks.build_walks(cl)
    for k in ("epi_index", "epi_disp", "epj_disp", "spj_disp", "id_epj", "id_spj"):
        np.testing.assert_array_equal(getattr(dev, k), getattr(host, k), err_msg=k)


def _cluster(pos, theta=0.3, n_leaf=20, n_group=512, r_out=0.01):
    n = len(pos)
    rng = np.random.default_rng(n)
    return ics.Cluster(pos=np.ascontiguousarray(pos, dtype=np.float64), vel=rng.normal(size=(n, 3)) * 0.1,
                       mass=np.full(n, 1.0 / n), r_out=r_out, r_in=0.1 * r_out, r_search=np.full(n, 1.5 * r_out),
                       theta=theta, n_leaf_limit=n_leaf, n_group_limit=n_group)


def _edge_cases():
    rng = np.random.default_rng(77)
    yield "single", _cluster(np.array([[0.1, -0.2, 0.3]]))
    yield "two_coincident", _cluster(np.array([[0.5, 0.5, 0.5], [0.5, 0.5, 0.5]]))
    # more coincident particles than a leaf holds: the cells split down to
    # level 21 and the deepest cell stays a leaf above n_leaf_limit
    yield "coincident_50_plus_field", _cluster(np.vstack([np.tile([[0.25, 0.25, 0.25]], (50, 1)),
                                                          rng.normal(size=(500, 3))]))
    yield "line", _cluster(np.column_stack([np.linspace(-1, 1, 3000), np.zeros(3000), np.zeros(3000)]))
    yield "leaf1_group1", _cluster(rng.normal(size=(700, 3)), n_leaf=1, n_group=1)
    yield "leaf8_group16", _cluster(rng.normal(size=(5000, 3)), n_leaf=8, n_group=16, theta=0.5)


@pytest.mark.parametrize("name", ["single", "two_coincident", "coincident_50_plus_field", "line", "leaf1_group1",
                                  "leaf8_group16"])
def test_device_lists_edge_cases(name):
    cl = dict(_edge_cases())[name]
    host = walks.build_walks(cl)
    with nbody.DeviceNBody(cl) as h:
        dev = h.lists()
        st = h.state()
    for k in ("epi_index", "epi_disp", "epj_disp", "spj_disp", "id_epj", "id_spj", "spj_mass", "spj_pos",
              "spj_quad"):
        np.testing.assert_array_equal(getattr(dev, k), getattr(host, k), err_msg=k)
    o = oracle.force(dev)
    idx = dev.epi_index
    np.testing.assert_array_equal(st["n_ngb"][idx], o["nnb"])
    ea = rel_err_vec(st["acc"][idx], o["acc"])
    ep = rel_err(st["pot"][idx], o["pot"])
    # coincident pairs have zero separation: the cutoff makes them finite
    assert np.isfinite(st["acc"]).all() and np.isfinite(st["pot"]).all()
    # Degenerate geometries: on the line the net force on most particles is a
    # near cancellation of its two sides, which multiplies relative errors,
    # so these cases use a looser bound than the cluster configurations.
    assert np.median(ea) <= 10 * MIXED_MEDIAN and np.median(ep) <= MIXED_MEDIAN, (np.median(ea), np.median(ep))
