"""The allocation-free entry point pgf_force_device_noalloc.

It serves callers that own all device memory themselves (one arena sized at
start-up, no cudaMalloc or cudaFree inside their step loop).  Here the test
plays that caller: it places the inputs and outputs in device memory itself
(through torch) and calls the entry point twice in a row through the C ABI.
Both calls must match the FP64 oracle within the mixed-precision tolerances of
the parity tests (counts exact) and agree with the regular dispatch/retrieve
path, which also shows that the shared static scratch is cleared between
calls.  Rows that no walk covers keep what the caller put there, and the
second call leaves the device's free memory unchanged.
"""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import oracle
from helpers import load_golden, rel_err, rel_err_vec, stats
from petar_gb300 import gpuforce, ics, walks

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
EPJ_DEV = np.dtype([("pos", "<f8", 3), ("mass", "<f4"), ("r_search2", "<f4")])
SPJ_DEV = np.dtype([("pos", "<f8", 3), ("mass", "<f4"), ("pad0", "<f4"), ("quad_traceless", "<f4", 6),
                    ("trace", "<f4"), ("pad1", "<f4")])
MIXED_MEDIAN, MIXED_P999, MIXED_MAX = 1e-6, 1e-5, 1e-3


def max_walks() -> int:
    text = (ROOT / "include" / "petar_gpuforce.h").read_text()
    return int(re.search(r"#define\s+PGF_NOALLOC_MAX_WALKS\s+(\d+)", text).group(1))


def _lib():
    lib = gpuforce.load()
    f = lib.pgf_force_device_noalloc
    vp, i64, cd = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double
    f.argtypes = [ctypes.c_int, vp, vp, i64, vp, vp, i64, vp, i64, vp, i64, vp, i64, cd, cd, cd, vp, vp, vp,
                  ctypes.c_char_p, ctypes.c_size_t]
    f.restype = ctypes.c_int
    return f


def _walk_table(wb, walks_kept):
    w = np.asarray(walks_kept, np.int64)
    return np.stack([wb.epi_disp[w], wb.n_epi[w], wb.epj_disp[w], wb.n_epj[w], wb.spj_disp[w], wb.n_spj[w]],
                    axis=1).astype(np.int64)


def _device_inputs(torch, wb, walks_kept=None):
    """The caller's own device copies of one multi-walk problem, in the
    documented device formats."""
    epi = np.concatenate([wb.epi_pos, wb.epi_rs[:, None]], axis=1)
    epj = np.zeros(wb.epj_mass.size, EPJ_DEV)
    epj["pos"] = wb.epj_pos
    epj["mass"] = wb.epj_mass.astype(np.float32)
    epj["r_search2"] = (wb.epj_rs * wb.epj_rs).astype(np.float32)
    q = wb.spj_quad
    tr = q[:, 0] + q[:, 1] + q[:, 2]
    spj = np.zeros(wb.spj_mass.size, SPJ_DEV)
    spj["pos"] = wb.spj_pos
    spj["mass"] = wb.spj_mass.astype(np.float32)
    spj["quad_traceless"] = np.stack([3.0 * q[:, 0] - tr, 3.0 * q[:, 1] - tr, 3.0 * q[:, 2] - tr,
                                      3.0 * q[:, 3], 3.0 * q[:, 4], 3.0 * q[:, 5]], axis=1).astype(np.float32)
    spj["trace"] = tr.astype(np.float32)
    table = _walk_table(wb, np.arange(wb.n_walk) if walks_kept is None else walks_kept)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).cuda()
    ni = wb.epi_rs.size
    return dict(epi=dev(epi), epj=dev(epj), epj_rs=dev(wb.epj_rs.astype(np.float64)), spj=dev(spj),
                id_epj=dev(wb.id_epj.astype(np.int32)), id_spj=dev(wb.id_spj.astype(np.int32)), table=dev(table),
                n_table=table.shape[0],
                accp=torch.empty((ni, 4), dtype=torch.float64, device="cuda"),
                nnb=torch.empty((ni,), dtype=torch.int32, device="cuda"))


def _call(f, torch, wb, d, n_walk=None, free_before_after=None):
    """One call with the outputs filled with NaN / -1 beforehand."""
    d["accp"].fill_(float("nan"))
    d["nnb"].fill_(-1)
    msg = ctypes.create_string_buffer(256)
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    if free_before_after is not None:
        free_before_after.append(torch.cuda.mem_get_info()[0])
    rc = f(d["n_table"] if n_walk is None else n_walk, d["table"].data_ptr(), d["epi"].data_ptr(), wb.epi_rs.size,
           d["epj"].data_ptr(), d["epj_rs"].data_ptr(), wb.epj_mass.size, d["spj"].data_ptr(), wb.spj_mass.size,
           d["id_epj"].data_ptr(), wb.id_epj.size, d["id_spj"].data_ptr(), wb.id_spj.size, wb.eps2, wb.rcut2,
           wb.G, d["accp"].data_ptr(), d["nnb"].data_ptr(), stream or None, msg, len(msg))
    torch.cuda.synchronize()
    if free_before_after is not None:
        free_before_after.append(torch.cuda.mem_get_info()[0])
    return rc, msg.value.decode(), d["accp"].cpu().numpy(), d["nnb"].cpu().numpy()


def _check(acc, pot, nnb, ref):
    np.testing.assert_array_equal(nnb, ref["nnb"])
    for e in (rel_err_vec(acc, ref["acc"]), rel_err(pot, ref["pot"])):
        s = stats(e)
        assert s["median"] <= MIXED_MEDIAN and s["p999"] <= MIXED_P999 and s["max"] <= MIXED_MAX, s


@pytest.mark.parametrize("case", ["plummer2048_walks", "binaries"])
def test_noalloc_matches_oracle_twice(case):
    torch = pytest.importorskip("torch")
    if case == "binaries":
        wb = walks.build_walks(ics.make_plummer_cluster(17, 8192, 0.01, binary_fraction=0.5))
    else:
        wb, _ = load_golden(case)
    o = oracle.force(wb)
    regular = gpuforce.compute(wb, gpuforce.PGF_PRECISION_MIXED)
    f = _lib()
    d = _device_inputs(torch, wb)
    free = []
    for k in range(2):
        rc, msg, accp, nnb = _call(f, torch, wb, d, free_before_after=free if k == 1 else None)
        assert rc == 0, msg
        _check(accp[:, :3], accp[:, 3], nnb, o)
        _check(accp[:, :3], accp[:, 3], nnb, regular)
    # The second call (kernels already loaded) takes no device memory.
    assert free[0] == free[1], free


def test_noalloc_leaves_uncovered_rows_untouched():
    torch = pytest.importorskip("torch")
    wb, _ = load_golden("plummer2048_walks")
    kept = np.array([w for w in range(wb.n_walk) if w % 3 != 1])
    gap = np.concatenate([np.arange(wb.epi_disp[w], wb.epi_disp[w + 1]) for w in range(wb.n_walk) if w % 3 == 1])
    covered = np.setdiff1d(np.arange(wb.epi_rs.size), gap)
    assert gap.size > 0
    o = oracle.force(wb)
    f = _lib()
    d = _device_inputs(torch, wb, kept)
    for _ in range(2):
        rc, msg, accp, nnb = _call(f, torch, wb, d)
        assert rc == 0, msg
        assert np.isnan(accp[gap]).all() and (nnb[gap] == -1).all()
        _check(accp[covered, :3], accp[covered, 3], nnb[covered],
               dict(acc=o["acc"][covered], pot=o["pot"][covered], nnb=o["nnb"][covered]))


def test_noalloc_rejects_too_many_walks():
    torch = pytest.importorskip("torch")
    wb, _ = load_golden("kernel_test")
    f = _lib()
    d = _device_inputs(torch, wb)
    rc, msg, _, nnb = _call(f, torch, wb, d, n_walk=max_walks() + 1)
    assert rc == 5 and "at most" in msg  # PGF_ERR_CAPACITY
    assert (nnb == -1).all()


def test_noalloc_rejects_out_of_range_ids_and_rows():
    torch = pytest.importorskip("torch")
    wb, _ = load_golden("kernel_test")
    wb.id_epj = wb.id_epj.copy()
    wb.id_epj[7] = wb.epj_mass.size
    f = _lib()
    d = _device_inputs(torch, wb)
    rc, msg, _, nnb = _call(f, torch, wb, d)
    assert rc == 1 and "EPJ id" in msg  # PGF_ERR_ARG, found by the device-side check
    assert (nnb == -1).all()
    # A table row whose offset is near INT64_MAX must not wrap past the check.
    wb2, _ = load_golden("kernel_test")
    d2 = _device_inputs(torch, wb2)
    table = _walk_table(wb2, np.arange(wb2.n_walk))
    table[0, 2] = np.iinfo(np.int64).max - 2
    d2["table"] = torch.from_numpy(table.view(np.uint8).reshape(-1)).cuda()
    rc, msg, _, nnb = _call(f, torch, wb2, d2)
    assert rc == 1 and "walk table row" in msg
    assert (nnb == -1).all()
