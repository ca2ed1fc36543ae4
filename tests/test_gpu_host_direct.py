"""Host-direct data movement (pgf_set_host_direct): the GPU reads the caller's
records and id lists in place in host memory and writes results straight into
the caller's Force records.  Every case runs twice, host-direct and with the
host packing into pinned staging, and the results must be bit-identical (the
gather kernels repeat the host packing's arithmetic), then meet the oracle."""
import ctypes

import numpy as np
import pytest

import oracle
from helpers import assert_mixed_parity, load_golden
from petar_gb300 import gpuforce, ics, walks
from petar_gb300.gpuforce import PGF_PRECISION_FP64, PGF_PRECISION_MIXED

pytestmark = pytest.mark.gpu


def both(fn):
    out = {}
    try:
        for hd in (False, True):
            gpuforce.set_host_direct(hd)
            out[hd] = fn()
    finally:
        gpuforce.set_host_direct(True)
    return out[False], out[True]


def assert_same(a: dict, b: dict):
    assert a.keys() == b.keys()
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_host_direct_active_on_this_device():
    gpuforce.CalcForceWithLinearCutoffCUDAMultiWalk(0, 0.0, 1e-4, 1.0)
    assert gpuforce.host_direct_active(), "the device does not report pageable memory access"


@pytest.mark.parametrize("precision", [PGF_PRECISION_MIXED, PGF_PRECISION_FP64])
@pytest.mark.parametrize("case", ["plummer2048_walks", "kernel_test_rsvar", "binaries65k"])
def test_same_as_staged(case, precision):
    if case == "binaries65k":  # 556-walk class dispatch: split walks, single launch
        wb = walks.build_walks(ics.make_plummer_cluster(41, 40000, 0.006, binary_fraction=0.5))
    else:
        wb, _ = load_golden(case)
    a, b = both(lambda: gpuforce.compute(wb, precision))
    assert_same(a, b)
    if precision == PGF_PRECISION_MIXED:
        assert_mixed_parity(b["acc"], b["pot"], b["nnb"], oracle.force(wb), label=case)


def test_same_as_staged_pipelined_and_ragged():
    """A pipelined dispatch keeps the host packing for the walks; the send
    and the stage-by-stage scatter of the results are host-direct."""
    wb = walks.build_walks(ics.make_plummer_cluster(23, 30000, 0.004, binary_fraction=0.5))
    gpuforce.set_dispatch_stages(3)
    try:
        a, b = both(lambda: gpuforce.compute(wb, PGF_PRECISION_MIXED))
    finally:
        gpuforce.set_dispatch_stages(0)
    assert_same(a, b)
    from test_gpu_parity import _ragged_batch
    rg = _ragged_batch()
    a, b = both(lambda: gpuforce.compute(rg, PGF_PRECISION_MIXED))
    assert_same(a, b)


def test_same_as_staged_modes():
    cl = ics.make_plummer_cluster(33, 20000, 0.004, binary_fraction=0.5)
    wb, co = walks.make_changeover(walks.build_walks(cl), cl.r_in, cl.r_out, seed=4)
    assert_same(*both(lambda: gpuforce.compute_changeover(wb, co)))
    acc = oracle.force(wb)["acc"]
    assert_same(*both(lambda: gpuforce.compute_gradient(wb, acc, acc)))
    rec = gpuforce.Records(wb)
    rec.force["acc"] = 5.0
    n = both(lambda: gpuforce.search_neighbors(wb, rec))
    np.testing.assert_array_equal(n[0], n[1])
    assert (rec.force["acc"] == 5.0).all()  # search mode writes n_ngb only


def test_non_index_dispatch_and_int32_counts():
    """The per-walk-array dispatch, and Force records with a 4-byte n_ngb
    between other fields: the scatter writes exactly the layout's fields."""
    wb, _ = load_golden("plummer2048_walks")
    rec = gpuforce.Records(wb)
    force_dt = np.dtype([("tag", "<i4"), ("n_ngb", "<i4"), ("acc", "<f8", 3), ("guard", "<f8"), ("pot", "<f8")],
                        align=True)
    epi = [rec.epi[wb.epi_disp[w]:wb.epi_disp[w + 1]] for w in range(wb.n_walk)]
    epj = [rec.epj[wb.id_epj[wb.epj_disp[w]:wb.epj_disp[w + 1]]] for w in range(wb.n_walk)]
    spj = [rec.spj[wb.id_spj[wb.spj_disp[w]:wb.spj_disp[w + 1]]] for w in range(wb.n_walk)]

    def run():
        f = gpuforce.CalcForceWithLinearCutoffCUDA(0, wb.eps2, wb.rcut2, wb.G)
        f(1, wb.n_walk, epi, rec.n_epi, epj, rec.n_epj, spj, rec.n_spj)
        force = [np.zeros(n, force_dt) for n in rec.n_epi]
        for x in force:
            x["tag"] = 77
            x["guard"] = -9.0
        gpuforce.RetrieveForceCUDA(1, wb.n_walk, rec.n_epi, force, force_dtype=force_dt)
        return np.concatenate(force)

    a, b = both(run)
    for k in force_dt.names:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert (b["tag"] == 77).all() and (b["guard"] == -9.0).all()
    assert_mixed_parity(b["acc"], b["pot"], b["n_ngb"], oracle.force(wb), label="non-index int32")


def test_bad_id_rejected_before_any_force_kernel():
    wb, _ = load_golden("plummer2048_walks")
    bad = wb.id_epj.copy()
    bad[wb.epj_disp[5] + 3] = wb.epj_mass.size
    good = wb.id_epj
    try:
        wb.id_epj = bad
        with pytest.raises(gpuforce.GpuForceError) as e:
            gpuforce.compute(wb)
        assert e.value.code == 1 and "walk 5" in str(e.value)
    finally:
        wb.id_epj = good
    res = gpuforce.compute(wb)
    assert_mixed_parity(res["acc"], res["pot"], res["nnb"], oracle.force(wb), label="after bad id")


def test_packed_records_take_the_host_path():
    """Packed record types (FP64 fields at 4-byte offsets) are not read or
    written in place by the GPU: send, dispatch and retrieve fall back to the
    host packing, and the results equal the staged path's bit for bit."""
    wb = walks.build_walks(ics.make_plummer_cluster(41, 40000, 0.006, binary_fraction=0.5))
    epi_dt = np.dtype([("tag", "<i4"), ("id", "<i8"), ("pos", "<f8", 3), ("r_search", "<f8")])
    epj_dt = np.dtype([("tag", "<i4"), ("id", "<i8"), ("mass", "<f8"), ("pos", "<f8", 3), ("r_search", "<f8")])
    spj_dt = np.dtype([("tag", "<i4"), ("mass", "<f8"), ("pos", "<f8", 3), ("quad", "<f8", 6)])
    force_dt = np.dtype([("tag", "<i4"), ("acc", "<f8", 3), ("pot", "<f8"), ("n_ngb", "<i8")])
    assert epi_dt.fields["pos"][1] % 8 and force_dt.fields["acc"][1] % 8
    ni = wb.epi_rs.size
    epi = np.zeros(ni, epi_dt)
    epi["pos"], epi["r_search"], epi["id"] = wb.epi_pos, wb.epi_rs, np.arange(ni)
    epj = np.zeros(wb.epj_mass.size, epj_dt)
    epj["mass"], epj["pos"], epj["r_search"] = wb.epj_mass, wb.epj_pos, wb.epj_rs
    spj = np.zeros(wb.spj_mass.size, spj_dt)
    spj["mass"], spj["pos"], spj["quad"] = wb.spj_mass, wb.spj_pos, wb.spj_quad
    id_epj = np.ascontiguousarray(wb.id_epj, np.int32)
    id_spj = np.ascontiguousarray(wb.id_spj, np.int32)
    n_epi = np.diff(wb.epi_disp).astype(np.int32)
    n_epj = np.diff(wb.epj_disp).astype(np.int32)
    n_spj = np.diff(wb.spj_disp).astype(np.int32)
    p_epi = [epi[wb.epi_disp[w]:wb.epi_disp[w + 1]] for w in range(wb.n_walk)]
    p_id_epj = [id_epj[wb.epj_disp[w]:wb.epj_disp[w + 1]] for w in range(wb.n_walk)]
    p_id_spj = [id_spj[wb.spj_disp[w]:wb.spj_disp[w + 1]] for w in range(wb.n_walk)]

    def run():
        f = gpuforce.CalcForceWithLinearCutoffCUDAMultiWalk(0, wb.eps2, wb.rcut2, wb.G)
        f(0, 0, None, None, None, None, None, None, epj, epj.size, spj, spj.size, True)
        f(0, wb.n_walk, p_epi, n_epi, p_id_epj, n_epj, p_id_spj, n_spj, epj, epj.size, spj, spj.size, False)
        force = np.zeros(ni, force_dt)
        force["tag"] = 31
        parts = [force[wb.epi_disp[w]:wb.epi_disp[w + 1]] for w in range(wb.n_walk)]
        gpuforce.RetrieveForceCUDA(0, wb.n_walk, n_epi, parts, force_dtype=force_dt)
        return force

    a, b = both(run)
    for k in force_dt.names:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert (b["tag"] == 31).all()
    assert_mixed_parity(b["acc"], b["pot"], b["n_ngb"], oracle.force(wb), label="packed records")
