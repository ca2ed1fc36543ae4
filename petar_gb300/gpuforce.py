"""ctypes binding of the soft-force C ABI (include/petar_gpuforce.h).

The classes mirror the reference functor pair so that Python callers and the
tests read like PeTar's own kernel test (src/simd_test.cxx:133-157):

* ``CalcForceWithLinearCutoffCUDAMultiWalk(rank, eps2, rcut2, G)`` and its
  ``__call__(tag, n_walk, epi, n_epi, id_epj, n_epj, id_spj, n_spj, epj,
  n_epj_tot, spj, n_spj_tot, send_flag)`` -- src/force_gpu_cuda.hpp:103-133;
* ``CalcForceWithLinearCutoffCUDA`` -- src/force_gpu_cuda.hpp:137-162;
* ``RetrieveForceCUDA(tag, n_walk, ni, force)`` -- src/force_gpu_cuda.hpp:165-168.

Particle records are numpy structured arrays with PeTar's field layout
(``EPI_DTYPE``, ``EPJ_DTYPE``, ``SPJ_DTYPE``, ``FORCE_DTYPE``); per-walk
arguments are lists of arrays (or of views into one array).  Errors raise
``GpuForceError`` carrying the library's status code and message.  There is no
CPU fallback: without the compiled library or a GPU every call fails.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PGF_OK = 0
PGF_PRECISION_MIXED = 0
PGF_PRECISION_FP64 = 1
NUM_KERNEL_VARIANTS = 9  # PGF_NUM_KERNEL_VARIANTS
DEFAULT_KERNEL_VARIANT = 7  # PGF_DEFAULT_KERNEL_VARIANT
PGF_MODE_FORCE = 0
PGF_MODE_NEIGHBOR_SEARCH = 1
PGF_MODE_FORCE_CHANGEOVER = 2
PGF_MODE_GRADIENT = 3

# PeTar's EPISoft (src/soft_ptcl.hpp:271-308): id, pos, r_search, rank_org, type.
EPI_DTYPE = np.dtype([("id", "<i8"), ("pos", "<f8", 3), ("r_search", "<f8"), ("rank_org", "<i4"),
                      ("type", "<i4")], align=True)
# PeTar's EPJSoft (src/soft_ptcl.hpp:311-376); group_data is a 16-byte union.
EPJ_DTYPE = np.dtype([("id", "<i8"), ("mass", "<f8"), ("pos", "<f8", 3), ("vel", "<f8", 3),
                      ("r_in", "<f8"), ("r_out", "<f8"), ("r_search", "<f8"), ("r_scale_next", "<f8"),
                      ("group_data", "<i8", 2), ("rank_org", "<i4"), ("adr_org", "<i4")], align=True)
# FDPS SPJQuadrupole-like superparticle: mass, pos, quad (xx, yy, zz, xy, xz, yz).
SPJ_DTYPE = np.dtype([("mass", "<f8"), ("pos", "<f8", 3), ("quad", "<f8", 6)], align=True)
# PeTar's ForceSoft (src/soft_ptcl.hpp:4-24): acc, pot, n_ngb.
FORCE_DTYPE = np.dtype([("acc", "<f8", 3), ("pot", "<f8"), ("n_ngb", "<i8")], align=True)
# For the fused changeover mode: EPISoft extended with the particle's changeover
# radii and self-potential mass, ForceSoft with the soft potential.  EPJSoft
# already carries id, r_in, r_out and group_data = (mass_backup, status).
EPI_CO_DTYPE = np.dtype([("id", "<i8"), ("pos", "<f8", 3), ("r_search", "<f8"), ("rank_org", "<i4"),
                         ("type", "<i4"), ("r_in", "<f8"), ("r_out", "<f8"), ("self_mass", "<f8")], align=True)
FORCE_CO_DTYPE = np.dtype([("acc", "<f8", 3), ("pot", "<f8"), ("n_ngb", "<i8"), ("pot_soft", "<f8")],
                          align=True)
# KDKDK_4TH builds of PeTar: EPISoft and EPJSoft carry acc, ForceSoft acorr
# (src/soft_ptcl.hpp:4-30, 271-345).
EPI_GR_DTYPE = np.dtype([("id", "<i8"), ("pos", "<f8", 3), ("r_search", "<f8"), ("rank_org", "<i4"),
                         ("type", "<i4"), ("acc", "<f8", 3)], align=True)
EPJ_GR_DTYPE = np.dtype([("id", "<i8"), ("mass", "<f8"), ("pos", "<f8", 3), ("vel", "<f8", 3),
                         ("acc", "<f8", 3), ("r_in", "<f8"), ("r_out", "<f8"), ("r_search", "<f8"),
                         ("r_scale_next", "<f8"), ("group_data", "<i8", 2), ("rank_org", "<i4"),
                         ("adr_org", "<i4")], align=True)
FORCE_GR_DTYPE = np.dtype([("acc", "<f8", 3), ("pot", "<f8"), ("acorr", "<f8", 3), ("n_ngb", "<i8")],
                          align=True)


class GpuForceError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"petar_gpuforce error {code}: {message}")
        self.code = code


class _EpiLayout(ctypes.Structure):
    _fields_ = [("size", ctypes.c_size_t), ("off_pos", ctypes.c_size_t), ("off_r_search", ctypes.c_size_t)]


class _EpjLayout(ctypes.Structure):
    _fields_ = [("size", ctypes.c_size_t), ("off_mass", ctypes.c_size_t), ("off_pos", ctypes.c_size_t),
                ("off_r_search", ctypes.c_size_t)]


class _SpjLayout(ctypes.Structure):
    _fields_ = [("size", ctypes.c_size_t), ("off_mass", ctypes.c_size_t), ("off_pos", ctypes.c_size_t),
                ("off_quad", ctypes.c_size_t), ("has_quad", ctypes.c_int)]


class _ChangeoverLayout(ctypes.Structure):
    _fields_ = [(k, ctypes.c_size_t) for k in (
        "epi_off_id", "epi_off_r_in", "epi_off_r_out", "epi_off_self_mass", "epj_off_id", "epj_off_r_in",
        "epj_off_r_out", "epj_off_mass_backup", "epj_off_status", "force_off_pot_soft")]


class _GradientLayout(ctypes.Structure):
    _fields_ = [("epi_off_acc", ctypes.c_size_t), ("epj_off_acc", ctypes.c_size_t),
                ("force_off_acorr", ctypes.c_size_t)]


class _ForceLayout(ctypes.Structure):
    _fields_ = [("size", ctypes.c_size_t), ("off_acc", ctypes.c_size_t), ("off_pot", ctypes.c_size_t),
                ("off_n_ngb", ctypes.c_size_t), ("n_ngb_bytes", ctypes.c_int)]


class Profile(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("copy", "send", "recv", "calc", "calc_main", "last_calc",
                                               "last_calc_main")] + \
               [(k, ctypes.c_int64) for k in ("n_walk", "n_epi", "n_epj", "n_spj", "n_call", "n_retest")]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def _layouts(epi_dt=EPI_DTYPE, epj_dt=EPJ_DTYPE, spj_dt=SPJ_DTYPE, force_dt=FORCE_DTYPE):
    el = _EpiLayout(epi_dt.itemsize, epi_dt.fields["pos"][1], epi_dt.fields["r_search"][1])
    jl = _EpjLayout(epj_dt.itemsize, epj_dt.fields["mass"][1], epj_dt.fields["pos"][1],
                    epj_dt.fields["r_search"][1])
    has_q = "quad" in spj_dt.fields
    sl = _SpjLayout(spj_dt.itemsize, spj_dt.fields["mass"][1], spj_dt.fields["pos"][1],
                    spj_dt.fields["quad"][1] if has_q else 0, 1 if has_q else 0)
    nb = force_dt.fields["n_ngb"][0].itemsize
    fl = _ForceLayout(force_dt.itemsize, force_dt.fields["acc"][1], force_dt.fields["pot"][1],
                      force_dt.fields["n_ngb"][1], nb)
    return el, jl, sl, fl


_LIB = None
_LIB_PATH: Path | None = None


def library_path() -> Path:
    return Path(__file__).resolve().parent / "lib" / "libpetar_gpuforce.so"


def load(build: bool = True) -> ctypes.CDLL:
    """Loads (building first if needed) the compiled library."""
    global _LIB, _LIB_PATH
    if _LIB is not None:
        return _LIB
    path = library_path()
    override = os.environ.get("PETAR_GPUFORCE_LIB")
    if override:
        path, build = Path(override), False
    if build:
        from .build import build_gpuforce
        path = build_gpuforce()
    if not path.exists():
        raise GpuForceError(-1, f"compiled library missing: {path}")
    lib = ctypes.CDLL(str(path))
    vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    sig = {
        "pgf_initialize": [ci, cd, cd, cd],
        "pgf_set_precision": [ci],
        "pgf_set_stream": [vp],
        "pgf_dispatch_index": [ci, ci, vp, vp, vp, vp, vp, vp, vp, vp, ci, vp, vp, ci, vp, ci],
        "pgf_dispatch": [ci, ci, vp, vp, vp, vp, vp, vp, vp, vp, vp],
        "pgf_retrieve": [ci, ci, vp, vp, vp],
        "pgf_set_walk_rcut2": [vp, ci],
        "pgf_recompute": [ci],
        "pgf_set_kernel_variant": [ci],
        "pgf_set_dispatch_stages": [ci],
        "pgf_set_walk_split": [ci],
        "pgf_set_walk_split_unit": [ci],
        "pgf_set_gradient_accuracy": [ci],
        "pgf_set_host_direct": [ci],
        "pgf_set_wait_limit_ns": [ctypes.c_uint64],
        "pgf_test_stall_producer": [ci],
        "pgf_get_host_direct": [vp],
        "pgf_set_mode": [ci],
        "pgf_set_changeover_layout": [vp],
        "pgf_set_gradient_layout": [vp],
        "pgf_get_kernel_variant": [vp],
        "pgf_autotune": [ci, ci, vp, vp],
        "pgf_autotune_dispatch": [ci, ci, vp, vp, vp, vp, vp, vp, vp, vp, vp, ci, vp, vp, vp],
        "pgf_wait": [ci],
        "pgf_get_profile": [vp],
        "pgf_clear_profile": [],
        "pgf_finalize": [],
    }
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = ci
    lib.pgf_last_error.argtypes = []
    lib.pgf_last_error.restype = ctypes.c_char_p
    _LIB = lib
    _LIB_PATH = path
    return lib


def _check(code: int) -> None:
    if code != PGF_OK:
        msg = load(build=False).pgf_last_error().decode(errors="replace")
        raise GpuForceError(code, msg)


def _ptrs(arrays) -> np.ndarray:
    return np.array([0 if a is None or a.size == 0 else a.ctypes.data for a in arrays], dtype=np.uint64)


def _ptr(a) -> int | None:
    return None if a is None else a.ctypes.data


def _ptr_table(arrays) -> np.ndarray:
    """Per-walk pointer table: a uint64 array of addresses is used as is, a
    list of per-walk arrays is converted."""
    if isinstance(arrays, np.ndarray) and arrays.dtype == np.uint64:
        return np.ascontiguousarray(arrays)
    if isinstance(arrays, (list, tuple)):
        return _ptrs(arrays)
    raise TypeError("expected a list of per-walk arrays or a uint64 pointer table")


def set_precision(precision: int) -> None:
    _check(load().pgf_set_precision(precision))


def set_stream(stream_handle: int | None) -> None:
    _check(load().pgf_set_stream(stream_handle or None))


def set_walk_rcut2(walk_rcut2: np.ndarray | None) -> None:
    if walk_rcut2 is None:
        _check(load().pgf_set_walk_rcut2(None, 0))
    else:
        a = np.ascontiguousarray(walk_rcut2, dtype=np.float64)
        _check(load().pgf_set_walk_rcut2(a.ctypes.data, a.size))


def set_kernel_variant(variant: int) -> None:
    _check(load().pgf_set_kernel_variant(variant))


def set_mode(mode: int) -> None:
    """PGF_MODE_FORCE (default) or PGF_MODE_NEIGHBOR_SEARCH for later dispatches."""
    _check(load().pgf_set_mode(mode))


def set_dispatch_stages(stages: int) -> None:
    """Pipeline stages of index dispatches (0: by size, 1: none, 2..8: forced)."""
    _check(load().pgf_set_dispatch_stages(stages))


def set_walk_split(enable: bool) -> None:
    """Split the most expensive walks of small single-launch dispatches over
    several CTAs (default on)."""
    _check(load().pgf_set_walk_split(1 if enable else 0))


def set_walk_split_unit(div: int) -> None:
    """Split walks costing more than 1/div of one SM's even share (default 16)."""
    _check(load().pgf_set_walk_split_unit(div))


def set_gradient_accuracy(mode: int) -> None:
    """Gradient pass far pairs: 1 compensated r^2 and 1/r (default), 0 FP32."""
    _check(load().pgf_set_gradient_accuracy(mode))


def set_host_direct(enable: bool) -> None:
    """Move data host-direct where the device supports it (default on): the
    GPU reads the caller's records in place and writes results into them."""
    _check(load().pgf_set_host_direct(1 if enable else 0))


def set_wait_limit_ns(limit_ns: int) -> None:
    """Limit of the kernels' bounded waits (0: the default, 1 s)."""
    _check(load().pgf_set_wait_limit_ns(int(limit_ns)))


def test_stall_producer(items: int) -> None:
    """Failure-detection test hook: the producer stops after `items` ring items."""
    _check(load().pgf_test_stall_producer(int(items)))


def host_direct_active() -> bool:
    v = ctypes.c_int(0)
    _check(load().pgf_get_host_direct(ctypes.byref(v)))
    return bool(v.value)


def get_kernel_variant() -> int:
    v = ctypes.c_int()
    _check(load().pgf_get_kernel_variant(ctypes.byref(v)))
    return v.value


def autotune(tag: int = 0, repeats: int = 3) -> tuple[int, float]:
    """Times every kernel variant on the tag's resident data; keeps the fastest."""
    v, ms = ctypes.c_int(), ctypes.c_double()
    _check(load().pgf_autotune(tag, repeats, ctypes.byref(v), ctypes.byref(ms)))
    return v.value, ms.value


def recompute(tag: int = 0) -> None:
    _check(load().pgf_recompute(tag))


def wait(tag: int = 0) -> None:
    _check(load().pgf_wait(tag))


def get_profile() -> dict:
    p = Profile()
    _check(load().pgf_get_profile(ctypes.byref(p)))
    return p.as_dict()


def clear_profile() -> None:
    _check(load().pgf_clear_profile())


def finalize() -> None:
    if _LIB is not None:
        _check(_LIB.pgf_finalize())


class CalcForceWithLinearCutoffCUDAMultiWalk:
    """Index-list dispatch functor (src/force_gpu_cuda.hpp:103-133)."""

    def __init__(self, rank: int = 0, eps2: float = 0.0, rcut2: float = 0.0, G: float = 1.0):
        self.initialize(rank, eps2, rcut2, G)

    def initialize(self, rank: int, eps2: float, rcut2: float, G: float) -> None:
        self.my_rank, self.eps2, self.rcut2, self.G = rank, eps2, rcut2, G
        _check(load().pgf_initialize(rank, eps2, rcut2, G))

    def __call__(self, tag, n_walk, epi, n_epi, id_epj, n_epj, id_spj, n_spj, epj, n_epj_tot, spj,
                 n_spj_tot, send_flag, epi_dtype=None):
        """epi_dtype: the EPI record type when ``epi`` is a table of raw
        addresses (default EPI_DTYPE, or the dtype of the arrays passed)."""
        lib = load()
        # Re-assert this functor's constants: like the reference, the device
        # state is process-wide and the last initialize() wins.
        _check(lib.pgf_initialize(self.my_rank, self.eps2, self.rcut2, self.G))
        if epi_dtype is None:
            epi_dtype = epi[0].dtype if isinstance(epi, (list, tuple)) and len(epi) else EPI_DTYPE
        el, jl, sl, _ = _layouts(epi_dtype, epj.dtype if epj is not None else EPJ_DTYPE,
                                 spj.dtype if spj is not None else SPJ_DTYPE)
        if send_flag:
            _check(lib.pgf_dispatch_index(tag, 0, None, None, None, None, None, None, None,
                                          _ptr(epj), int(n_epj_tot), ctypes.byref(jl), _ptr(spj),
                                          int(n_spj_tot), ctypes.byref(sl), 1))
            return 0
        n_epi = np.ascontiguousarray(n_epi, dtype=np.int32)
        n_epj = np.ascontiguousarray(n_epj, dtype=np.int32)
        n_spj = np.ascontiguousarray(n_spj, dtype=np.int32)
        pe, pj, ps = (_ptr_table(a) for a in (epi, id_epj, id_spj))
        _check(lib.pgf_dispatch_index(tag, int(n_walk), _ptr(pe), _ptr(n_epi), ctypes.byref(el), _ptr(pj),
                                      _ptr(n_epj), _ptr(ps), _ptr(n_spj), None, 0, None, None, 0, None, 0))
        return 0


class CalcForceWithLinearCutoffCUDA:
    """Per-walk EPJ/SPJ array dispatch functor (src/force_gpu_cuda.hpp:137-162)."""

    def __init__(self, rank: int = 0, eps2: float = 0.0, rcut2: float = 0.0, G: float = 1.0):
        self.initialize(rank, eps2, rcut2, G)

    def initialize(self, rank, eps2, rcut2, G):
        self.my_rank, self.eps2, self.rcut2, self.G = rank, eps2, rcut2, G
        _check(load().pgf_initialize(rank, eps2, rcut2, G))

    def __call__(self, tag, n_walk, epi, n_epi, epj, n_epj, spj, n_spj):
        lib = load()
        _check(lib.pgf_initialize(self.my_rank, self.eps2, self.rcut2, self.G))
        def dt(a, default):
            return a[0].dtype if isinstance(a, (list, tuple)) and len(a) else default
        el, jl, sl, _ = _layouts(dt(epi, EPI_DTYPE), dt(epj, EPJ_DTYPE), dt(spj, SPJ_DTYPE))
        n_epi = np.ascontiguousarray(n_epi, dtype=np.int32)
        n_epj = np.ascontiguousarray(n_epj, dtype=np.int32)
        n_spj = np.ascontiguousarray(n_spj, dtype=np.int32)
        # The pointer tables must stay referenced until the call returns.
        pe, pj, ps = _ptr_table(epi), _ptr_table(epj), _ptr_table(spj)
        _check(lib.pgf_dispatch(tag, int(n_walk), _ptr(pe), _ptr(n_epi), ctypes.byref(el), _ptr(pj), _ptr(n_epj),
                                ctypes.byref(jl), _ptr(ps), _ptr(n_spj), ctypes.byref(sl)))
        return 0


def RetrieveForceCUDA(tag, n_walk, ni, force, force_dtype=None) -> int:
    """src/force_gpu_cuda.hpp:165-168: overwrites acc, pot, n_ngb of force[w].
    force_dtype: the record type when ``force`` is a table of raw addresses."""
    lib = load()
    fdt = force_dtype
    if fdt is None:
        fdt = force[0].dtype if isinstance(force, (list, tuple)) and len(force) else FORCE_DTYPE
    _, _, _, fl = _layouts(force_dt=fdt)
    ni = np.ascontiguousarray(ni, dtype=np.int32)
    pf = _ptr_table(force)
    _check(lib.pgf_retrieve(tag, int(n_walk), _ptr(ni), _ptr(pf), ctypes.byref(fl)))
    return 0


# ---------------------------------------------------------------------------
# Convenience layer over WalkBatch (petar_gb300.walks)


class Records:
    """A WalkBatch converted to PeTar-layout record arrays plus the per-walk
    pointer tables the functors take."""

    def __init__(self, batch, co=None, acc=None):
        """co: a walks.ChangeoverSet for the fused changeover mode (extended
        EPI and Force records; EPJ ids, radii and group_data filled in).
        acc: (epi_acc, epj_acc) for the KDKDK_4TH gradient mode (records of a
        KDKDK_4TH build)."""
        ni = batch.epi_rs.size
        gr = acc is not None
        self.epi = np.zeros(ni, EPI_CO_DTYPE if co is not None else (EPI_GR_DTYPE if gr else EPI_DTYPE))
        self.epi["pos"] = batch.epi_pos
        self.epi["r_search"] = batch.epi_rs
        self.epi["type"] = 1
        self.epi["id"] = np.arange(ni)
        self.epj = np.zeros(batch.epj_mass.size, EPJ_GR_DTYPE if gr else EPJ_DTYPE)
        self.epj["mass"] = batch.epj_mass
        self.epj["pos"] = batch.epj_pos
        self.epj["r_search"] = batch.epj_rs
        self.epj["id"] = np.arange(batch.epj_mass.size)
        self.co = co
        if gr:
            self.epi["acc"] = acc[0]
            self.epj["acc"] = acc[1]
        if co is not None:
            self.epi["id"] = co.epi_id
            self.epi["r_in"] = co.epi_r_in
            self.epi["r_out"] = co.epi_r_out
            self.epi["self_mass"] = co.epi_self_mass
            self.epj["id"] = co.epj_id
            self.epj["r_in"] = co.epj_r_in
            self.epj["r_out"] = co.epj_r_out
            gd = self.epj["group_data"].view(np.float64).reshape(-1, 2)
            gd[:, 0] = co.epj_mass_backup
            gd[:, 1] = co.epj_status
            self.epj["group_data"] = gd.view(np.int64).reshape(-1, 2)
        self.spj = np.zeros(batch.spj_mass.size, SPJ_DTYPE)
        self.spj["mass"] = batch.spj_mass
        self.spj["pos"] = batch.spj_pos
        self.spj["quad"] = batch.spj_quad
        self.force = np.zeros(ni, FORCE_CO_DTYPE if co is not None else (FORCE_GR_DTYPE if gr else FORCE_DTYPE))
        self.id_epj = np.ascontiguousarray(batch.id_epj, dtype=np.int32)
        self.id_spj = np.ascontiguousarray(batch.id_spj, dtype=np.int32)
        self.n_walk = batch.n_walk
        self.n_epi = np.diff(batch.epi_disp).astype(np.int32)
        self.n_epj = np.diff(batch.epj_disp).astype(np.int32)
        self.n_spj = np.diff(batch.spj_disp).astype(np.int32)
        isz, fsz = self.epi.dtype.itemsize, self.force.dtype.itemsize
        d = np.asarray(batch.epi_disp[:-1], dtype=np.uint64)
        self.p_epi = (np.uint64(self.epi.ctypes.data) + d * np.uint64(isz)).astype(np.uint64)
        self.p_force = (np.uint64(self.force.ctypes.data) + d * np.uint64(fsz)).astype(np.uint64)
        self.p_id_epj = (np.uint64(self.id_epj.ctypes.data if self.id_epj.size else 0)
                         + np.asarray(batch.epj_disp[:-1], np.uint64) * np.uint64(4)).astype(np.uint64)
        self.p_id_spj = (np.uint64(self.id_spj.ctypes.data if self.id_spj.size else 0)
                         + np.asarray(batch.spj_disp[:-1], np.uint64) * np.uint64(4)).astype(np.uint64)
        self.walk_rcut2 = batch.walk_rcut2
        self.eps2, self.rcut2, self.G = batch.eps2, batch.rcut2, batch.G


def autotune_dispatch(rec: Records, tag: int = 0, repeats: int = 2) -> dict:
    """Tunes the dispatch pipeline's stage count and the walk-split unit on
    the caller's records (send first), through pgf_autotune_dispatch."""
    send_j(rec, tag)
    el, _, _, fl = _layouts(epi_dt=rec.epi.dtype, force_dt=rec.force.dtype)
    st, sp, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    set_walk_rcut2(rec.walk_rcut2)
    try:
        _check(load().pgf_autotune_dispatch(tag, rec.n_walk, _ptr(rec.p_epi), _ptr(rec.n_epi), ctypes.byref(el),
                                            _ptr(rec.p_id_epj), _ptr(rec.n_epj), _ptr(rec.p_id_spj),
                                            _ptr(rec.n_spj), _ptr(rec.p_force), ctypes.byref(fl), int(repeats),
                                            ctypes.byref(st), ctypes.byref(sp), ctypes.byref(ms)))
    finally:
        set_walk_rcut2(None)
    return {"stages": st.value, "split_unit": sp.value, "ms": ms.value}


def send_j(rec: Records, tag: int = 0) -> None:
    f = CalcForceWithLinearCutoffCUDAMultiWalk(0, rec.eps2, rec.rcut2, rec.G)
    f(tag, 0, None, None, None, None, None, None, rec.epj, rec.epj.size, rec.spj, rec.spj.size, True)


def dispatch(rec: Records, tag: int = 0, send: bool = True) -> None:
    """One multi-walk force call: send_flag=true then false, as FDPS does."""
    f = CalcForceWithLinearCutoffCUDAMultiWalk(0, rec.eps2, rec.rcut2, rec.G)
    if send:
        f(tag, 0, None, None, None, None, None, None, rec.epj, rec.epj.size, rec.spj, rec.spj.size, True)
    set_walk_rcut2(rec.walk_rcut2)
    try:
        f(tag, rec.n_walk, rec.p_epi, rec.n_epi, rec.p_id_epj, rec.n_epj, rec.p_id_spj, rec.n_spj,
          None, 0, None, 0, False, epi_dtype=rec.epi.dtype)
    finally:
        set_walk_rcut2(None)


def retrieve(rec: Records, tag: int = 0) -> np.ndarray:
    RetrieveForceCUDA(tag, rec.n_walk, rec.n_epi, rec.p_force, force_dtype=rec.force.dtype)
    return rec.force


def compute(batch, precision: int = PGF_PRECISION_MIXED, rec: Records | None = None) -> dict:
    """acc, pot, nnb for every EPI row of a WalkBatch through the C ABI."""
    rec = rec if rec is not None else Records(batch)
    set_precision(precision)
    dispatch(rec)
    f = retrieve(rec)
    return dict(acc=f["acc"].copy(), pot=f["pot"].copy(), nnb=f["n_ngb"].copy())


def search_neighbors(batch, rec: Records | None = None) -> np.ndarray:
    """n_ngb of every EPI row of a WalkBatch in neighbour-search mode
    (SearchNeighborEpEpNoSimd semantics: no softening in the test, SPJ lists
    ignored).  acc and pot of the records are left as they were."""
    rec = rec if rec is not None else Records(batch)
    set_mode(PGF_MODE_NEIGHBOR_SEARCH)
    try:
        dispatch(rec)
        f = retrieve(rec)
    finally:
        set_mode(PGF_MODE_FORCE)
    return f["n_ngb"].copy()


def changeover_layout(rec: Records) -> _ChangeoverLayout:
    """The pgf_changeover_layout of a Records built with a ChangeoverSet."""
    fi, fj, ff = rec.epi.dtype.fields, rec.epj.dtype.fields, rec.force.dtype.fields
    gd = fj["group_data"][1]
    return _ChangeoverLayout(fi["id"][1], fi["r_in"][1], fi["r_out"][1], fi["self_mass"][1], fj["id"][1],
                             fj["r_in"][1], fj["r_out"][1], gd, gd + 8, ff["pot_soft"][1])


def set_changeover_layout(rec: Records | None) -> None:
    """Sets (rec with a ChangeoverSet) or clears (None) the changeover layout."""
    if rec is None:
        _check(load().pgf_set_changeover_layout(None))
    else:
        lay = changeover_layout(rec)
        _check(load().pgf_set_changeover_layout(ctypes.byref(lay)))


def compute_changeover(batch, co, rec: Records | None = None) -> dict:
    """acc, pot (total), pot_soft and nnb of every EPI row in the fused
    changeover mode, through the C ABI (send and dispatch as FDPS does)."""
    rec = rec if rec is not None else Records(batch, co)
    set_precision(PGF_PRECISION_MIXED)
    set_changeover_layout(rec)
    set_mode(PGF_MODE_FORCE_CHANGEOVER)
    try:
        dispatch(rec)
        f = retrieve(rec)
    finally:
        set_mode(PGF_MODE_FORCE)
        set_changeover_layout(None)
    return dict(acc=f["acc"].copy(), pot=f["pot"].copy(), pot_soft=f["pot_soft"].copy(), nnb=f["n_ngb"].copy())


def set_gradient_layout(rec: Records | None) -> None:
    """Sets (rec built with accelerations) or clears (None) the gradient layout."""
    if rec is None:
        _check(load().pgf_set_gradient_layout(None))
        return
    lay = _GradientLayout(rec.epi.dtype.fields["acc"][1], rec.epj.dtype.fields["acc"][1],
                          rec.force.dtype.fields["acorr"][1])
    _check(load().pgf_set_gradient_layout(ctypes.byref(lay)))


def compute_gradient(batch, epi_acc, epj_acc, rec: Records | None = None) -> dict:
    """acorr, acc and pot of every EPI row from the KDKDK_4TH gradient pass
    through the C ABI."""
    rec = rec if rec is not None else Records(batch, acc=(epi_acc, epj_acc))
    set_gradient_layout(rec)
    set_mode(PGF_MODE_GRADIENT)
    try:
        dispatch(rec)
        f = retrieve(rec)
    finally:
        set_mode(PGF_MODE_FORCE)
        set_gradient_layout(None)
    return dict(acorr=f["acorr"].copy(), acc=f["acc"].copy(), pot=f["pot"].copy(), nnb=f["n_ngb"].copy())
