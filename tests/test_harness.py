"""The interaction-list builder (the FDPS stand-in) and the initial conditions."""
import numpy as np
import pytest

import oracle
from petar_gb300 import ics, walks


@pytest.fixture(scope="module")
def c1():
    cl = ics.make_plummer_cluster(1, 2048, 0.02, theta=0.3)
    return cl, walks.build_walks(cl)


def test_groups_partition_particles(c1):
    cl, wb = c1
    assert wb.epi_disp[0] == 0 and wb.epi_disp[-1] == cl.n
    assert (np.diff(wb.epi_disp) > 0).all()
    assert (np.diff(wb.epi_disp) <= cl.n_group_limit).all()
    assert np.array_equal(np.sort(wb.epi_index), np.arange(cl.n))


def test_list_counts_equal_global_counts(c1):
    """Symmetric-search opening with the full r_search puts every pair with
    |xi - xj| < max(rs_i, rs_j) into the walk's EPJ list, so per-list neighbour
    counts equal a global N^2 count."""
    cl, wb = c1
    per_list = oracle.force(wb)["nnb"]
    glob = oracle.nnb_global(cl.pos, cl.r_search)[wb.epi_index]
    np.testing.assert_array_equal(per_list, glob)


def test_list_counts_equal_global_counts_variable_rs():
    cl = ics.make_plummer_cluster(7, 3000, 0.02, theta=0.5, n_group_limit=64)
    rng = np.random.default_rng(3)
    cl.r_search = cl.r_out * (1.0 + 2.0 * rng.random(cl.n))
    wb = walks.build_walks(cl)
    np.testing.assert_array_equal(oracle.force(wb)["nnb"], oracle.nnb_global(cl.pos, cl.r_search)[wb.epi_index])


def test_each_particle_is_epj_or_inside_one_spj(c1):
    """Every particle contributes to every walk exactly once: as an EPJ or
    through exactly one SPJ (cell) that contains it."""
    cl, wb = c1
    # mass seen by each walk = total mass
    for w in range(wb.n_walk):
        ej = wb.id_epj[wb.epj_disp[w]:wb.epj_disp[w + 1]]
        sj = wb.id_spj[wb.spj_disp[w]:wb.spj_disp[w + 1]]
        assert np.unique(ej).size == ej.size
        m = wb.epj_mass[ej].sum() + wb.spj_mass[sj].sum()
        assert abs(m - 1.0) < 1e-12


def test_tree_force_close_to_direct(c1):
    """theta = 0.3 with quadrupoles: tree force within 1e-2 of the direct sum
    (median far below)."""
    cl, wb = c1
    o = oracle.force(wb)
    targets = wb.epi_index[::16]
    rows = np.arange(0, wb.epi_rs.size, 16)
    acc, pot = oracle.direct(cl.pos, cl.mass, targets, wb.eps2, wb.rcut2)
    err = np.linalg.norm(o["acc"][rows] - acc, axis=1) / np.linalg.norm(acc, axis=1)
    assert np.median(err) < 2e-3
    assert err.max() < 5e-2


def test_plummer_henon_units():
    cl = ics.make_plummer_cluster(5, 20000, 0.01)
    assert abs(cl.mass.sum() - 1.0) < 1e-12
    ke = 0.5 * (cl.mass * (cl.vel ** 2).sum(1)).sum()
    assert 0.2 < ke < 0.3  # virial equilibrium: K = -E = 1/4


def test_kroupa_range_and_slope():
    rng = np.random.default_rng(0)
    m = ics.kroupa_masses(rng, 200000)
    assert m.min() >= 0.08 and m.max() <= 150.0
    frac_low = (m < 0.5).mean()
    assert 0.6 < frac_low < 0.8


def test_binaries_bound_and_separated():
    cl = ics.make_plummer_cluster(9, 4000, 0.003, binary_fraction=0.5)
    assert cl.n == 6000
    n_single = 2000
    p1, p2 = cl.pos[n_single::2], cl.pos[n_single + 1::2]
    sep = np.linalg.norm(p1 - p2, axis=1)
    assert sep.min() > 0 and sep.max() < 2 * 1e-2 * 1.01


def test_subset_and_concat_roundtrip(c1):
    _, wb = c1
    sub = wb.subset(np.array([3, 0, 5]))
    assert sub.n_walk == 3
    o_full = oracle.force(wb)
    o_sub = oracle.force(sub)
    rows = np.concatenate([np.arange(wb.epi_disp[w], wb.epi_disp[w + 1]) for w in (3, 0, 5)])
    np.testing.assert_array_equal(o_sub["acc"], o_full["acc"][rows])
    both = walks.concat_batches([wb, wb])
    o2 = oracle.force(both)
    np.testing.assert_array_equal(o2["nnb"][:wb.epi_rs.size], o_full["nnb"])
    np.testing.assert_array_equal(o2["acc"][wb.epi_rs.size:], o_full["acc"])
