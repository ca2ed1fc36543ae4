"""FP64 CPU oracle for the soft-force path (test infrastructure only).

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package; the product never does.  ``oracle.c``
restates the reference's FP64 functors (src/soft_force.hpp:38-87, 160-200)
with the GPU functor's neighbour test (src/force_gpu_cuda.cu:62-64).  Parity of
this restatement is pinned against the reference's own functors through the
fixtures in ``tests/golden`` (made by ``tests/golden/make_golden.py`` from
libraries that ``oracle/ref/build_ref.sh`` compiles out of the reference
sources).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_LIB = None


def build(force: bool = False) -> Path:
    out = HERE / "liboracle.so"
    src = HERE / "oracle.c"
    if force or not out.exists() or out.stat().st_mtime < src.stat().st_mtime:
        tmp = out.with_suffix(".so.tmp")
        subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                        "-fno-fast-math", str(src), "-o", str(tmp), "-lm"], check=True)
        os.replace(tmp, out)
    return out


REF_DIR = HERE / "_ref"


def build_ref_gpu_driver(force: bool = False) -> Path | None:
    """Compiles ref/ref_gpu_driver.cu (this project's host driver for the
    reference's own CUDA kernels) into _ref/libref_gpu_driver.so; None without
    nvcc."""
    import shutil
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        return None
    REF_DIR.mkdir(exist_ok=True)
    out = REF_DIR / "libref_gpu_driver.so"
    src = HERE / "ref" / "ref_gpu_driver.cu"
    if force or not out.exists() or out.stat().st_mtime < src.stat().st_mtime:
        tmp = out.with_suffix(".so.tmp")
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-Xcompiler",
                        "-fPIC", "-shared", str(src), "-o", str(tmp), "-lcuda"], check=True)
        os.replace(tmp, out)
    return out


_REF_GPU = None


class ReferenceKernelUnavailable(RuntimeError):
    pass


def ref_gpu(batch, repeats: int = 0) -> dict:
    """The reference's own CUDA kernels (force_kernel_ep_ep + force_kernel_ep_sp
    of src/force_gpu_cuda.cu, from _ref/ref_force_gpu.cubin) on a WalkBatch:
    acc, pot and nnb as its retrieve writes them (FP32 widened to FP64), and
    ms, the mean time of `repeats` re-runs of the two kernels."""
    global _REF_GPU
    cubin = REF_DIR / "ref_force_gpu.cubin"
    if not cubin.exists():
        raise ReferenceKernelUnavailable("the reference's kernels were not compiled (no reference sources here)")
    if _REF_GPU is None:
        lib = ctypes.CDLL(str(build_ref_gpu_driver()))
        vp = ctypes.c_void_p
        lib.ref_gpu_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
        lib.ref_gpu_load.restype = ctypes.c_int
        lib.ref_gpu_force.argtypes = ([ctypes.c_int] + [vp] * 7 + [ctypes.c_int64] + [vp] * 3 + [ctypes.c_int64]
                                      + [vp] * 3 + [ctypes.c_double] * 3 + [ctypes.c_int] + [vp] * 4
                                      + [ctypes.c_char_p, ctypes.c_size_t])
        lib.ref_gpu_force.restype = ctypes.c_int
        msg = ctypes.create_string_buffer(256)
        if lib.ref_gpu_load(str(cubin).encode(), msg, len(msg)) != 0:
            raise ReferenceKernelUnavailable(msg.value.decode())
        _REF_GPU = lib
    a = [_c(batch.epi_disp, np.int64), _c(batch.epi_pos, np.float64), _c(batch.epi_rs, np.float64),
         _c(batch.epj_disp, np.int64), _c(batch.id_epj, np.int32), _c(batch.spj_disp, np.int64),
         _c(batch.id_spj, np.int32)]
    j = [_c(batch.epj_pos, np.float64), _c(batch.epj_mass, np.float64), _c(batch.epj_rs, np.float64)]
    sp = [_c(batch.spj_pos, np.float64), _c(batch.spj_mass, np.float64), _c(batch.spj_quad, np.float64)]
    ni = batch.epi_rs.size
    out = dict(acc=np.zeros((ni, 3)), pot=np.zeros(ni), nnb=np.zeros(ni, np.int64))
    ms = ctypes.c_double(0.0)
    msg = ctypes.create_string_buffer(256)
    rc = _REF_GPU.ref_gpu_force(batch.n_walk, *[_p(x) for x in a], batch.epj_mass.size, *[_p(x) for x in j],
                                batch.spj_mass.size, *[_p(x) for x in sp], float(batch.eps2), float(batch.rcut2),
                                float(batch.G), int(repeats), _p(out["acc"]), _p(out["pot"]), _p(out["nnb"]),
                                ctypes.byref(ms), msg, len(msg))
    if rc != 0:
        raise RuntimeError(f"reference kernels: {msg.value.decode()} ({rc})")
    out["ms"] = ms.value
    return out


def _lib():
    global _LIB
    if _LIB is None:
        lib = ctypes.CDLL(str(build()))
        vp = ctypes.c_void_p
        lib.oracle_force.restype = None
        lib.oracle_force.argtypes = [ctypes.c_int64] + [vp] * 13 + [ctypes.c_double] * 3 + [vp, ctypes.c_int] + [vp] * 7
        lib.oracle_nnb_global.restype = None
        lib.oracle_nnb_global.argtypes = [ctypes.c_int64, vp, vp, ctypes.c_double, vp]
        lib.oracle_direct.restype = None
        lib.oracle_direct.argtypes = [ctypes.c_int64, vp, ctypes.c_int64, vp, vp] + [ctypes.c_double] * 3 + [vp, vp]
        lib.oracle_co_w.restype = None
        lib.oracle_co_w.argtypes = [ctypes.c_int64] + [vp] * 5
        lib.oracle_co_w_two.restype = None
        lib.oracle_co_w_two.argtypes = [ctypes.c_int64] + [vp] * 7
        lib.oracle_gradient.restype = None
        lib.oracle_gradient.argtypes = [ctypes.c_int64] + [vp] * 13 + [ctypes.c_double] * 3 + [vp] * 4
        lib.oracle_force_changeover.restype = None
        lib.oracle_force_changeover.argtypes = ([ctypes.c_int64] + [vp] * 13 + [ctypes.c_double] * 3 + [vp]
                                                + [vp] * 9 + [vp] * 4)
        _LIB = lib
    return _LIB


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a):
    return None if a is None else a.ctypes.data


def force(batch, nnb_with_eps: bool = True, parts: bool = False) -> dict:
    """Oracle acc/pot/nnb for every EPI row of a WalkBatch (walk order)."""
    lib = _lib()
    ni = batch.epi_rs.size
    arrs = dict(
        epi_disp=_c(batch.epi_disp, np.int64), epi_pos=_c(batch.epi_pos, np.float64),
        epi_rs=_c(batch.epi_rs, np.float64), epj_pos=_c(batch.epj_pos, np.float64),
        epj_mass=_c(batch.epj_mass, np.float64), epj_rs=_c(batch.epj_rs, np.float64),
        spj_pos=_c(batch.spj_pos, np.float64), spj_mass=_c(batch.spj_mass, np.float64),
        spj_quad=_c(batch.spj_quad, np.float64), epj_disp=_c(batch.epj_disp, np.int64),
        id_epj=_c(batch.id_epj, np.int32), spj_disp=_c(batch.spj_disp, np.int64),
        id_spj=_c(batch.id_spj, np.int32))
    wr = None if batch.walk_rcut2 is None else _c(batch.walk_rcut2, np.float64)
    out = dict(acc=np.zeros((ni, 3)), pot=np.zeros(ni), nnb=np.zeros(ni, np.int64))
    if parts:
        out.update(acc_ep=np.zeros((ni, 3)), pot_ep=np.zeros(ni), acc_sp=np.zeros((ni, 3)),
                   pot_sp=np.zeros(ni))
    lib.oracle_force(batch.n_walk, *[_p(arrs[k]) for k in (
        "epi_disp", "epi_pos", "epi_rs", "epj_pos", "epj_mass", "epj_rs", "spj_pos", "spj_mass",
        "spj_quad", "epj_disp", "id_epj", "spj_disp", "id_spj")],
        float(batch.eps2), float(batch.rcut2), float(batch.G), _p(wr), int(bool(nnb_with_eps)),
        _p(out["acc"]), _p(out["pot"]), _p(out["nnb"]), _p(out.get("acc_ep")), _p(out.get("pot_ep")),
        _p(out.get("acc_sp")), _p(out.get("pot_sp")))
    return out


def co_w(r_in, r_out, dr):
    """(W_acc, W_pot) of changeovers (r_in, r_out) at separations dr
    (src/changeover.hpp:294-334)."""
    r_in, r_out, dr = (_c(a, np.float64) for a in (r_in, r_out, dr))
    a = np.zeros(dr.size)
    p = np.zeros(dr.size)
    _lib().oracle_co_w(dr.size, _p(r_in), _p(r_out), _p(dr), _p(a), _p(p))
    return a, p


def co_w_two(r_in1, r_out1, r_in2, r_out2, dr):
    """The pair forms: W of the changeover with the larger r_out."""
    arrs = [_c(a, np.float64) for a in (r_in1, r_out1, r_in2, r_out2, dr)]
    n = arrs[-1].size
    a = np.zeros(n)
    p = np.zeros(n)
    _lib().oracle_co_w_two(n, *[_p(x) for x in arrs], _p(a), _p(p))
    return a, p


def force_changeover(batch, co) -> dict:
    """acc, pot_tot, pot_soft and nnb of every EPI row with the changeover
    correction of its neighbours applied (see oracle_force_changeover).
    ``co`` holds per-EPI id, r_in, r_out, self_mass and per-EPJ id, r_in,
    r_out, mass_backup, status arrays (petar_gb300.walks.ChangeoverSet)."""
    lib = _lib()
    ni = batch.epi_rs.size
    arrs = [_c(batch.epi_disp, np.int64), _c(batch.epi_pos, np.float64), _c(batch.epi_rs, np.float64),
            _c(batch.epj_pos, np.float64), _c(batch.epj_mass, np.float64), _c(batch.epj_rs, np.float64),
            _c(batch.spj_pos, np.float64), _c(batch.spj_mass, np.float64), _c(batch.spj_quad, np.float64),
            _c(batch.epj_disp, np.int64), _c(batch.id_epj, np.int32), _c(batch.spj_disp, np.int64),
            _c(batch.id_spj, np.int32)]
    wr = None if batch.walk_rcut2 is None else _c(batch.walk_rcut2, np.float64)
    coa = [_c(co.epi_id, np.int64), _c(co.epi_r_in, np.float64), _c(co.epi_r_out, np.float64),
           _c(co.epi_self_mass, np.float64), _c(co.epj_id, np.int64), _c(co.epj_r_in, np.float64),
           _c(co.epj_r_out, np.float64), _c(co.epj_mass_backup, np.float64), _c(co.epj_status, np.float64)]
    out = dict(acc=np.zeros((ni, 3)), pot=np.zeros(ni), pot_soft=np.zeros(ni), nnb=np.zeros(ni, np.int64))
    lib.oracle_force_changeover(batch.n_walk, *[_p(a) for a in arrs], float(batch.eps2), float(batch.rcut2),
                                float(batch.G), _p(wr), *[_p(a) for a in coa], _p(out["acc"]), _p(out["pot"]),
                                _p(out["pot_soft"]), _p(out["nnb"]))
    return out


def gradient(batch, epi_acc, epj_acc) -> dict:
    """KDKDK_4TH gradient-correction pass of every EPI row (oracle_gradient):
    acorr, acc and pot as the reference's functors write them."""
    lib = _lib()
    ni = batch.epi_rs.size
    arrs = [_c(batch.epi_disp, np.int64), _c(batch.epi_pos, np.float64), _c(epi_acc, np.float64),
            _c(batch.epj_pos, np.float64), _c(batch.epj_mass, np.float64), _c(epj_acc, np.float64),
            _c(batch.spj_pos, np.float64), _c(batch.spj_mass, np.float64), _c(batch.spj_quad, np.float64),
            _c(batch.epj_disp, np.int64), _c(batch.id_epj, np.int32), _c(batch.spj_disp, np.int64),
            _c(batch.id_spj, np.int32)]
    wr = None if batch.walk_rcut2 is None else _c(batch.walk_rcut2, np.float64)
    out = dict(acorr=np.zeros((ni, 3)), acc=np.zeros((ni, 3)), pot=np.zeros(ni))
    lib.oracle_gradient(batch.n_walk, *[_p(a) for a in arrs], float(batch.eps2), float(batch.rcut2),
                        float(batch.G), _p(wr), _p(out["acorr"]), _p(out["acc"]), _p(out["pot"]))
    return out


def nnb_global(pos, rs, eps2: float = 0.0) -> np.ndarray:
    pos = _c(pos, np.float64)
    rs = _c(rs, np.float64)
    out = np.zeros(rs.size, np.int64)
    _lib().oracle_nnb_global(rs.size, _p(pos), _p(rs), float(eps2), _p(out))
    return out


def direct(pos, mass, targets, eps2: float, rcut2: float, G: float = 1.0):
    pos = _c(pos, np.float64)
    mass = _c(mass, np.float64)
    t = _c(targets, np.int64)
    acc = np.zeros((t.size, 3))
    pot = np.zeros(t.size)
    _lib().oracle_direct(t.size, _p(t), mass.size, _p(pos), _p(mass), float(eps2), float(rcut2),
                         float(G), _p(acc), _p(pot))
    return acc, pot
