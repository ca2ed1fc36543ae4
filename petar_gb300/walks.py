"""Interaction lists in the form the multi-walk dispatch functor receives them.

``build_walks`` runs the native interaction-list builder (the FDPS stand-in in
``csrc/harness/walk_builder.cpp``) over a cluster and returns a ``WalkBatch``:
the arguments of one ``CalcForceWithLinearCutoffCUDAMultiWalk`` call
(src/force_gpu_cuda.hpp:120-132) for all groups at once, as flat arrays:

* EPI: the i-particles of every walk, concatenated; walk ``w`` owns
  ``epi[epi_disp[w]:epi_disp[w+1]]`` (the reference passes ``epi[w]`` pointers
  and ``n_epi[w]``).
* EPJ / SPJ: the shared particle and superparticle arrays (``epj``,
  ``n_epj_tot``, ``spj``, ``n_spj_tot``).
* id lists: walk ``w`` interacts with ``epj[id_epj[epj_disp[w]:epj_disp[w+1]]]``
  and ``spj[id_spj[spj_disp[w]:spj_disp[w+1]]]``.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .ics import Cluster

_LIB = None


def _harness():
    global _LIB
    if _LIB is None:
        from .build import build_harness
        path = build_harness()
        lib = ctypes.CDLL(str(path))
        lib.pgfh_build.restype = ctypes.c_void_p
        lib.pgfh_build.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        lib.pgfh_fetch.restype = None
        lib.pgfh_fetch.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 10
        lib.pgfh_free.restype = None
        lib.pgfh_free.argtypes = [ctypes.c_void_p]
        _LIB = lib
    return _LIB


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


@dataclass
class WalkBatch:
    epi_pos: np.ndarray      # (ni, 3) float64
    epi_rs: np.ndarray       # (ni,)   float64
    epi_disp: np.ndarray     # (n_walk + 1,) int64
    epj_pos: np.ndarray      # (n_epj_tot, 3) float64
    epj_mass: np.ndarray     # (n_epj_tot,)
    epj_rs: np.ndarray       # (n_epj_tot,)
    spj_pos: np.ndarray      # (n_spj_tot, 3)
    spj_mass: np.ndarray     # (n_spj_tot,)
    spj_quad: np.ndarray     # (n_spj_tot, 6) xx, yy, zz, xy, xz, yz
    epj_disp: np.ndarray     # (n_walk + 1,) int64
    id_epj: np.ndarray       # int32
    spj_disp: np.ndarray     # (n_walk + 1,) int64
    id_spj: np.ndarray       # int32
    eps2: float
    rcut2: float
    G: float
    walk_rcut2: np.ndarray | None = None   # per-walk r_out^2 for ensembles
    epi_index: np.ndarray | None = None    # EPI row -> particle index of the input cluster(s)
    meta: dict = field(default_factory=dict)

    @property
    def n_walk(self) -> int:
        return self.epi_disp.size - 1

    @property
    def n_epi(self) -> np.ndarray:
        return np.diff(self.epi_disp)

    @property
    def n_epj(self) -> np.ndarray:
        return np.diff(self.epj_disp)

    @property
    def n_spj(self) -> np.ndarray:
        return np.diff(self.spj_disp)

    def interactions(self) -> tuple[int, int]:
        """(EP-EP, EP-SP) interaction counts: sum over walks of n_i * n_j."""
        ni = self.n_epi.astype(np.int64)
        return int((ni * self.n_epj).sum()), int((ni * self.n_spj).sum())

    def subset(self, walks: np.ndarray) -> "WalkBatch":
        """The same problem restricted to the given walks (j arrays shared)."""
        walks = np.asarray(walks, dtype=np.int64)
        ni = self.n_epi[walks]
        nej = self.n_epj[walks]
        nsj = self.n_spj[walks]
        epi_idx = np.concatenate([np.arange(self.epi_disp[w], self.epi_disp[w + 1]) for w in walks]) \
            if walks.size else np.zeros(0, np.int64)
        ej = np.concatenate([self.id_epj[self.epj_disp[w]:self.epj_disp[w + 1]] for w in walks]) \
            if walks.size else np.zeros(0, np.int32)
        sj = np.concatenate([self.id_spj[self.spj_disp[w]:self.spj_disp[w + 1]] for w in walks]) \
            if walks.size else np.zeros(0, np.int32)
        disp = lambda c: np.concatenate([[0], np.cumsum(c)]).astype(np.int64)
        return WalkBatch(
            epi_pos=self.epi_pos[epi_idx], epi_rs=self.epi_rs[epi_idx], epi_disp=disp(ni),
            epj_pos=self.epj_pos, epj_mass=self.epj_mass, epj_rs=self.epj_rs,
            spj_pos=self.spj_pos, spj_mass=self.spj_mass, spj_quad=self.spj_quad,
            epj_disp=disp(nej), id_epj=ej.astype(np.int32), spj_disp=disp(nsj),
            id_spj=sj.astype(np.int32), eps2=self.eps2, rcut2=self.rcut2, G=self.G,
            walk_rcut2=None if self.walk_rcut2 is None else self.walk_rcut2[walks],
            epi_index=None if self.epi_index is None else self.epi_index[epi_idx],
            meta=dict(self.meta))


def build_walks(cl: Cluster) -> WalkBatch:
    """Builds the tree and every group's interaction lists for one cluster."""
    lib = _harness()
    n = cl.n
    pos = np.ascontiguousarray(cl.pos, dtype=np.float64)
    mass = np.ascontiguousarray(cl.mass, dtype=np.float64)
    rs = np.ascontiguousarray(cl.r_search, dtype=np.float64)
    sizes = np.zeros(4, np.int64)
    h = lib.pgfh_build(n, _ptr(pos), _ptr(mass), _ptr(rs), float(cl.theta), int(cl.n_leaf_limit),
                       int(cl.n_group_limit), _ptr(sizes))
    if not h:
        raise ValueError("interaction-list builder rejected the input")
    ng, nc, ne, ns = (int(s) for s in sizes)
    order = np.empty(n, np.int64)
    gbeg = np.empty(ng + 1, np.int64)
    edisp = np.empty(ng + 1, np.int64)
    sdisp = np.empty(ng + 1, np.int64)
    id_epj = np.empty(ne, np.int32)
    id_spj = np.empty(ns, np.int32)
    cmass = np.empty(nc)
    cpos = np.empty((nc, 3))
    cquad = np.empty((nc, 6))
    clev = np.empty(nc, np.int32)
    try:
        lib.pgfh_fetch(h, _ptr(order), _ptr(gbeg), _ptr(edisp), _ptr(sdisp), _ptr(id_epj), _ptr(id_spj),
                       _ptr(cmass), _ptr(cpos), _ptr(cquad), _ptr(clev))
    finally:
        lib.pgfh_free(h)
    spos = pos[order]
    return WalkBatch(
        epi_pos=spos, epi_rs=rs[order], epi_disp=gbeg,
        epj_pos=spos.copy(), epj_mass=mass[order], epj_rs=rs[order].copy(),
        spj_pos=cpos, spj_mass=cmass, spj_quad=cquad,
        epj_disp=edisp, id_epj=id_epj, spj_disp=sdisp, id_spj=id_spj,
        eps2=cl.eps * cl.eps, rcut2=cl.r_out * cl.r_out, G=cl.G, epi_index=order,
        meta={"n": n, "n_cell": nc, "theta": cl.theta, "r_out": cl.r_out,
              "n_leaf_limit": cl.n_leaf_limit, "n_group_limit": cl.n_group_limit})


def concat_batches(batches: list[WalkBatch]) -> WalkBatch:
    """Joins independent clusters into one multi-walk problem: j arrays are
    concatenated, id lists offset, and each walk keeps its cluster's r_out^2."""
    e_off = np.cumsum([0] + [b.epj_mass.size for b in batches])
    s_off = np.cumsum([0] + [b.spj_mass.size for b in batches])
    i_off = np.cumsum([0] + [b.epi_rs.size for b in batches])

    def cat_disp(key):
        parts, base = [np.zeros(1, np.int64)], 0
        for b in batches:
            d = getattr(b, key)
            parts.append(d[1:] + base)
            base += int(d[-1])
        return np.concatenate(parts)

    walk_rcut2 = np.concatenate([
        (b.walk_rcut2 if b.walk_rcut2 is not None else np.full(b.n_walk, b.rcut2)) for b in batches])
    return WalkBatch(
        epi_pos=np.concatenate([b.epi_pos for b in batches]),
        epi_rs=np.concatenate([b.epi_rs for b in batches]),
        epi_disp=cat_disp("epi_disp"),
        epj_pos=np.concatenate([b.epj_pos for b in batches]),
        epj_mass=np.concatenate([b.epj_mass for b in batches]),
        epj_rs=np.concatenate([b.epj_rs for b in batches]),
        spj_pos=np.concatenate([b.spj_pos for b in batches]),
        spj_mass=np.concatenate([b.spj_mass for b in batches]),
        spj_quad=np.concatenate([b.spj_quad for b in batches]),
        epj_disp=cat_disp("epj_disp"),
        id_epj=np.concatenate([b.id_epj + np.int32(o) for b, o in zip(batches, e_off[:-1])]).astype(np.int32),
        spj_disp=cat_disp("spj_disp"),
        id_spj=np.concatenate([b.id_spj + np.int32(o) for b, o in zip(batches, s_off[:-1])]).astype(np.int32),
        eps2=batches[0].eps2, rcut2=float(walk_rcut2.max()) if walk_rcut2.size else 0.0,
        G=batches[0].G, walk_rcut2=walk_rcut2,
        epi_index=np.concatenate([(b.epi_index if b.epi_index is not None else np.arange(b.epi_rs.size)) + o
                                  for b, o in zip(batches, i_off[:-1])]),
        meta={"n_cluster": len(batches)})


@dataclass
class ChangeoverSet:
    """Per-particle changeover data for the fused changeover mode.

    PeTar's changeover radii scale with mass as r * max((m / m_avg)^(1/3), 1)
    (ChangeOver::setR, src/changeover.hpp:43-60); the artificial-particle
    information is the (mass_backup, status) pair of
    src/artificial_particles.hpp:15-90 (single: both 0; member: status < 0,
    potential mass in mass_backup, soft mass 0; anything else: its potential
    is removed from neighbours').  self_mass is the mass whose self-potential
    G m / r_out the correction removes (src/hard.hpp:1663-1674), 0 for none."""
    epi_id: np.ndarray
    epi_r_in: np.ndarray
    epi_r_out: np.ndarray
    epi_self_mass: np.ndarray
    epj_id: np.ndarray
    epj_r_in: np.ndarray
    epj_r_out: np.ndarray
    epj_mass_backup: np.ndarray
    epj_status: np.ndarray


def make_changeover(batch: WalkBatch, r_in: float, r_out: float, member_fraction: float = 0.1,
                    artificial_fraction: float = 0.05, seed: int = 0) -> tuple[WalkBatch, ChangeoverSet]:
    """Changeover data for a single-cluster batch (EPI and EPJ rows are the
    same particles, ``batch.epi_index``): mass-scaled radii, and a random share
    of members (soft mass 0, mass in mass_backup) and artificial particles.
    Returns the batch with the members' EPJ masses set to 0, and the set."""
    assert batch.epi_index is not None and batch.epi_rs.size == batch.epj_mass.size
    rng = np.random.default_rng(seed)
    n = batch.epj_mass.size
    ids = batch.epi_index.astype(np.int64)
    m = batch.epj_mass.astype(np.float64)
    m_fac = m / m.mean()
    scale = np.maximum(np.power(m_fac, 1.0 / 3.0), 1.0)  # std::pow(m_fac, 1.0/3.0) as setR
    u = rng.random(n)
    member = u < member_fraction
    artificial = (u >= member_fraction) & (u < member_fraction + artificial_fraction)
    status = np.zeros(n)
    status[member] = -1.0
    status[artificial] = 1.0
    mbk = np.zeros(n)
    mbk[member] = m[member]
    soft_m = np.where(member, 0.0, m)
    self_mass = np.where(member | artificial, 0.0, m)
    co = ChangeoverSet(epi_id=ids, epi_r_in=r_in * scale, epi_r_out=r_out * scale, epi_self_mass=self_mass,
                       epj_id=ids.copy(), epj_r_in=r_in * scale, epj_r_out=r_out * scale,
                       epj_mass_backup=mbk, epj_status=status)
    out = WalkBatch(**{k: getattr(batch, k) for k in batch.__dataclass_fields__})
    out.epj_mass = soft_m
    return out, co


def subset_changeover(batch: WalkBatch, co: ChangeoverSet, walks: np.ndarray) -> ChangeoverSet:
    """The changeover set of ``batch.subset(walks)``: EPI arrays restricted to
    the rows of those walks, EPJ arrays shared."""
    walks = np.asarray(walks, dtype=np.int64)
    rows = np.concatenate([np.arange(batch.epi_disp[w], batch.epi_disp[w + 1]) for w in walks]) \
        if walks.size else np.zeros(0, np.int64)
    return ChangeoverSet(epi_id=co.epi_id[rows], epi_r_in=co.epi_r_in[rows], epi_r_out=co.epi_r_out[rows],
                         epi_self_mass=co.epi_self_mass[rows], epj_id=co.epj_id, epj_r_in=co.epj_r_in,
                         epj_r_out=co.epj_r_out, epj_mass_backup=co.epj_mass_backup, epj_status=co.epj_status)
