"""The allocation-free entry point pgf_force_device_noalloc.

It serves callers that own all device memory themselves (one arena sized at
start-up, no cudaMalloc or cudaFree inside their step loop).  Here the test
plays that caller: it places the inputs and outputs in device memory itself
(through torch) and calls the entry point twice in a row through the C ABI.
Both calls must reproduce the regular dispatch/retrieve path within the
mixed-precision tolerances of the parity tests (counts exact), which also shows
that the shared static scratch is cleared between calls.
"""
import ctypes

import numpy as np
import pytest

from helpers import load_golden, rel_err, rel_err_vec, stats
from petar_gb300 import gpuforce, ics, walks

pytestmark = pytest.mark.gpu

PGF_NOALLOC_MAX_WALKS = 16384
EPJ_DEV = np.dtype([("pos", "<f8", 3), ("mass", "<f4"), ("r_search2", "<f4")])
SPJ_DEV = np.dtype([("pos", "<f8", 3), ("mass", "<f4"), ("pad0", "<f4"), ("quad_traceless", "<f4", 6),
                    ("trace", "<f4"), ("pad1", "<f4")])
MIXED_MEDIAN, MIXED_P999, MIXED_MAX = 1e-6, 1e-5, 1e-3


def _lib():
    lib = gpuforce.load()
    f = lib.pgf_force_device_noalloc
    vp, i64, cd = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double
    f.argtypes = [ctypes.c_int, vp, vp, i64, vp, vp, i64, vp, i64, vp, i64, vp, i64, cd, cd, cd, vp, vp, vp,
                  ctypes.c_char_p, ctypes.c_size_t]
    f.restype = ctypes.c_int
    return f


def _device_inputs(torch, wb):
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
    table = np.stack([wb.epi_disp[:-1], wb.n_epi, wb.epj_disp[:-1], wb.n_epj, wb.spj_disp[:-1], wb.n_spj],
                     axis=1).astype(np.int64)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).cuda()
    return dict(epi=dev(epi), epj=dev(epj), epj_rs=dev(wb.epj_rs.astype(np.float64)), spj=dev(spj),
                id_epj=dev(wb.id_epj.astype(np.int32)), id_spj=dev(wb.id_spj.astype(np.int32)), table=dev(table))


def _call(f, torch, wb, d, n_walk=None):
    ni = wb.epi_rs.size
    accp = torch.full((ni, 4), float("nan"), dtype=torch.float64, device="cuda")
    nnb = torch.full((ni,), -1, dtype=torch.int32, device="cuda")
    msg = ctypes.create_string_buffer(256)
    stream = torch.cuda.current_stream().cuda_stream
    rc = f(wb.n_walk if n_walk is None else n_walk, d["table"].data_ptr(), d["epi"].data_ptr(), ni,
           d["epj"].data_ptr(), d["epj_rs"].data_ptr(), wb.epj_mass.size, d["spj"].data_ptr(), wb.spj_mass.size,
           d["id_epj"].data_ptr(), wb.id_epj.size, d["id_spj"].data_ptr(), wb.id_spj.size, wb.eps2, wb.rcut2,
           wb.G, accp.data_ptr(), nnb.data_ptr(), stream or None, msg, len(msg))
    torch.cuda.synchronize()
    return rc, msg.value.decode(), accp.cpu().numpy(), nnb.cpu().numpy()


def _check_against_regular(res_acc, res_pot, res_nnb, ref):
    np.testing.assert_array_equal(res_nnb, ref["nnb"])
    for e in (rel_err_vec(res_acc, ref["acc"]), rel_err(res_pot, ref["pot"])):
        s = stats(e)
        assert s["median"] <= MIXED_MEDIAN and s["p999"] <= MIXED_P999 and s["max"] <= MIXED_MAX, s


@pytest.mark.parametrize("case", ["plummer2048_walks", "binaries"])
def test_noalloc_matches_regular_path_twice(case):
    torch = pytest.importorskip("torch")
    if case == "binaries":
        wb = walks.build_walks(ics.make_plummer_cluster(17, 8192, 0.01, binary_fraction=0.5))
    else:
        wb, _ = load_golden(case)
    ref = gpuforce.compute(wb, gpuforce.PGF_PRECISION_MIXED)
    f = _lib()
    d = _device_inputs(torch, wb)
    for _ in range(2):
        rc, msg, accp, nnb = _call(f, torch, wb, d)
        assert rc == 0, msg
        _check_against_regular(accp[:, :3], accp[:, 3], nnb, ref)


def test_noalloc_rejects_too_many_walks():
    torch = pytest.importorskip("torch")
    wb, _ = load_golden("kernel_test")
    f = _lib()
    d = _device_inputs(torch, wb)
    rc, msg, _, nnb = _call(f, torch, wb, d, n_walk=PGF_NOALLOC_MAX_WALKS + 1)
    assert rc == 5 and "at most" in msg  # PGF_ERR_CAPACITY
    assert (nnb == -1).all()


def test_noalloc_rejects_out_of_range_ids():
    torch = pytest.importorskip("torch")
    wb, _ = load_golden("kernel_test")
    wb.id_epj = wb.id_epj.copy()
    wb.id_epj[7] = wb.epj_mass.size
    f = _lib()
    d = _device_inputs(torch, wb)
    rc, msg, _, nnb = _call(f, torch, wb, d)
    assert rc == 1 and "EPJ id" in msg  # PGF_ERR_ARG, found by the device-side check
    assert (nnb == -1).all()
