"""ctypes binding of the device-resident tree step (``pgf_nbody_*`` in
include/petar_gpuforce.h).

``DeviceNBody(cluster)`` copies a cluster to the device, builds its tree and
interaction lists there and evaluates the soft force.  ``run(n_steps, dt)``
advances it by kick-drift-force-kick steps (PeTar's tree step for singles:
kickOne src/petar.hpp:1198-1212, driftSingle src/petar.hpp:1326-1340,
treeSoftForce src/petar.hpp:879-907), all of them captured in one CUDA graph
when ``graph=True``.  ``lists()`` returns the last build's tree and lists as a
``WalkBatch`` in the layout the host list builder (``walks.build_walks``)
produces, so the two can be compared entry for entry.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import gpuforce
from .ics import Cluster
from .walks import WalkBatch


class Config(ctypes.Structure):
    _fields_ = [("eps2", ctypes.c_double), ("r_out", ctypes.c_double), ("G", ctypes.c_double),
                ("theta", ctypes.c_double), ("n_leaf_limit", ctypes.c_int), ("n_group_limit", ctypes.c_int),
                ("precision", ctypes.c_int), ("kernel_variant", ctypes.c_int),
                ("list_capacity_factor", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in (
        "n_cells", "n_groups", "n_epj_entries", "n_spj_entries", "interactions_epep", "interactions_epsp",
        "total_epep", "total_epsp", "steps")] + \
        [("last_tree_ms", ctypes.c_double), ("last_force_ms", ctypes.c_double), ("kernel_variant", ctypes.c_int),
         ("cap_cells", ctypes.c_int), ("cap_epj_entries", ctypes.c_int64), ("cap_spj_entries", ctypes.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


# pgf_nbody_sample: one sampled particle at one force evaluation.
SAMPLE_DTYPE = np.dtype([("acc", "<f8", 3), ("pot", "<f8"), ("acc64", "<f8", 3), ("pot64", "<f8"),
                         ("n_ngb", "<i4"), ("n_ngb64", "<i4"), ("record", "<i4"), ("pad", "<i4")])
assert SAMPLE_DTYPE.itemsize == 80

_BOUND = False


def _lib() -> ctypes.CDLL:
    global _BOUND
    lib = gpuforce.load()
    if not _BOUND:
        vp, ci, cd, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int64
        sig = {
            "pgf_nbody_create": [vp, i64, vp, vp, vp, vp, vp],
            "pgf_nbody_force": [vp],
            "pgf_nbody_run": [vp, ci, cd, ci, vp],
            "pgf_nbody_get": [vp, vp, vp, vp, vp, vp],
            "pgf_nbody_set_state": [vp, vp, vp],
            "pgf_nbody_energy": [vp, vp, vp],
            "pgf_nbody_get_stats": [vp, vp],
            "pgf_nbody_export_lists": [vp] + [vp] * 10,
            "pgf_nbody_autotune": [vp, ci, vp, vp],
            "pgf_nbody_set_group_limit": [vp, ci],
            "pgf_nbody_autotune_groups": [vp, vp, ci, ci, vp, vp, vp, vp, vp],
            "pgf_nbody_set_sample": [vp, ci, vp, ci],
            "pgf_nbody_get_sample": [vp, vp, vp],
            "pgf_nbody_destroy": [vp],
        }
        for name, args in sig.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = ci
        lib.pgf_nbody_last_error.argtypes = []
        lib.pgf_nbody_last_error.restype = ctypes.c_char_p
        _BOUND = True
    return lib


def _check(code: int) -> None:
    if code != gpuforce.PGF_OK:
        raise gpuforce.GpuForceError(code, _lib().pgf_nbody_last_error().decode(errors="replace"))


def _p(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


class DeviceNBody:
    """Particles of one cluster resident on the current device."""

    def __init__(self, cl: Cluster, precision: int = gpuforce.PGF_PRECISION_MIXED, kernel_variant: int = -1,
                 list_capacity_factor: float = 2.0):
        lib = _lib()
        self.cluster = cl
        self.n = cl.n
        self.cfg = Config(cl.eps * cl.eps, cl.r_out, cl.G, cl.theta, cl.n_leaf_limit, cl.n_group_limit,
                          precision, kernel_variant, list_capacity_factor)
        pos = np.ascontiguousarray(cl.pos, dtype=np.float64)
        vel = np.ascontiguousarray(cl.vel, dtype=np.float64)
        mass = np.ascontiguousarray(cl.mass, dtype=np.float64)
        rs = np.ascontiguousarray(cl.r_search, dtype=np.float64)
        h = ctypes.c_void_p()
        _check(lib.pgf_nbody_create(ctypes.byref(self.cfg), self.n, _p(pos), _p(vel), _p(mass), _p(rs),
                                    ctypes.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib().pgf_nbody_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def force(self) -> None:
        _check(_lib().pgf_nbody_force(self._h))

    def run(self, n_steps: int, dt: float, graph: bool = True) -> float:
        """Advances n_steps steps; returns the device milliseconds of the run."""
        ms = ctypes.c_double()
        _check(_lib().pgf_nbody_run(self._h, int(n_steps), float(dt), 1 if graph else 0, ctypes.byref(ms)))
        return ms.value

    def state(self) -> dict:
        n = self.n
        out = {"pos": np.empty((n, 3)), "vel": np.empty((n, 3)), "acc": np.empty((n, 3)), "pot": np.empty(n),
               "n_ngb": np.empty(n, np.int32)}
        _check(_lib().pgf_nbody_get(self._h, _p(out["pos"]), _p(out["vel"]), _p(out["acc"]), _p(out["pot"]),
                                    _p(out["n_ngb"])))
        return out

    def set_state(self, pos: np.ndarray | None = None, vel: np.ndarray | None = None) -> None:
        pos = None if pos is None else np.ascontiguousarray(pos, dtype=np.float64)
        vel = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64)
        _check(_lib().pgf_nbody_set_state(self._h, _p(pos), _p(vel)))

    def energy(self) -> tuple[float, float]:
        k, p = ctypes.c_double(), ctypes.c_double()
        _check(_lib().pgf_nbody_energy(self._h, ctypes.byref(k), ctypes.byref(p)))
        return k.value, p.value

    def stats(self) -> dict:
        s = Stats()
        _check(_lib().pgf_nbody_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()

    def autotune(self, repeats: int = 3) -> tuple[int, float]:
        v, ms = ctypes.c_int(), ctypes.c_double()
        _check(_lib().pgf_nbody_autotune(self._h, repeats, ctypes.byref(v), ctypes.byref(ms)))
        return v.value, ms.value

    def set_group_limit(self, n_group_limit: int) -> None:
        """Rebuilds the tree and lists with this n_group_limit (and evaluates)."""
        _check(_lib().pgf_nbody_set_group_limit(self._h, int(n_group_limit)))

    def autotune_groups(self, limits=(256, 512, 1024, 2048), repeats: int = 2) -> dict:
        """Times tree + lists + force per evaluation for each n_group_limit
        candidate (kernel variant tuned per candidate) and keeps the fastest."""
        lim = np.ascontiguousarray(limits, dtype=np.int32)
        ms = np.zeros(lim.size)
        inter = np.zeros(lim.size, np.int64)
        best, var, bms = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _check(_lib().pgf_nbody_autotune_groups(self._h, _p(lim), lim.size, int(repeats), _p(ms), _p(inter),
                                                ctypes.byref(best), ctypes.byref(var), ctypes.byref(bms)))
        return {"best_n_group_limit": best.value, "kernel_variant": var.value, "best_ms": bms.value,
                "candidates": [{"n_group_limit": int(g), "ms_per_evaluation": float(t), "interactions": int(i),
                                "value": float(i) / (t * 1e-3) / 1e9 if t > 0 else None}
                               for g, t, i in zip(lim, ms, inter)]}

    def set_sample(self, particles: np.ndarray, max_records: int) -> None:
        """Record, after every force evaluation, the mixed-precision result of
        the given particles next to an FP64 evaluation over the same lists."""
        idx = np.ascontiguousarray(particles, dtype=np.int64)
        self._sample_n = idx.size
        self._sample_max = int(max_records)
        _check(_lib().pgf_nbody_set_sample(self._h, idx.size, _p(idx) if idx.size else None, int(max_records)))

    def samples(self) -> np.ndarray:
        """Records so far, shaped (evaluations, sampled particles)."""
        n = ctypes.c_int()
        out = np.zeros(self._sample_max * self._sample_n, SAMPLE_DTYPE)
        _check(_lib().pgf_nbody_get_sample(self._h, ctypes.byref(n), _p(out)))
        return out[:n.value * self._sample_n].reshape(n.value, self._sample_n)

    def lists(self) -> WalkBatch:
        """The last build as a WalkBatch over the current positions."""
        st = self.stats()
        ng, nc, ne, ns = st["n_groups"], st["n_cells"], st["n_epj_entries"], st["n_spj_entries"]
        order = np.empty(self.n, np.int64)
        gbeg = np.empty(ng + 1, np.int64)
        edisp = np.empty(ng + 1, np.int64)
        sdisp = np.empty(ng + 1, np.int64)
        id_epj = np.empty(ne, np.int32)
        id_spj = np.empty(ns, np.int32)
        cmass = np.empty(nc)
        cpos = np.empty((nc, 3))
        cquad = np.empty((nc, 6))
        clev = np.empty(nc, np.int32)
        _check(_lib().pgf_nbody_export_lists(self._h, _p(order), _p(gbeg), _p(edisp), _p(sdisp), _p(id_epj),
                                             _p(id_spj), _p(cmass), _p(cpos), _p(cquad), _p(clev)))
        s = self.state()
        cl = self.cluster
        spos = s["pos"][order]
        rs = np.ascontiguousarray(cl.r_search, dtype=np.float64)
        return WalkBatch(
            epi_pos=spos, epi_rs=rs[order], epi_disp=gbeg,
            epj_pos=spos.copy(), epj_mass=cl.mass[order], epj_rs=rs[order].copy(),
            spj_pos=cpos, spj_mass=cmass, spj_quad=cquad,
            epj_disp=edisp, id_epj=id_epj, spj_disp=sdisp, id_spj=id_spj,
            eps2=cl.eps * cl.eps, rcut2=cl.r_out * cl.r_out, G=cl.G, epi_index=order,
            meta={"n": self.n, "n_cell": nc, "theta": cl.theta, "r_out": cl.r_out, "cell_level": clev,
                  "n_leaf_limit": cl.n_leaf_limit, "n_group_limit": cl.n_group_limit})
