"""Shared helpers for the soft-force tests: golden fixtures as WalkBatch
objects and error statistics."""
from __future__ import annotations

from pathlib import Path

import numpy as np

from petar_gb300.walks import WalkBatch

GOLDEN = Path(__file__).resolve().parent / "golden"


def load_golden(name: str) -> tuple[WalkBatch, dict]:
    d = dict(np.load(GOLDEN / f"{name}.npz"))
    wb = WalkBatch(epi_pos=d["epi_pos"], epi_rs=d["epi_rs"], epi_disp=d["epi_disp"], epj_pos=d["epj_pos"],
                   epj_mass=d["epj_mass"], epj_rs=d["epj_rs"], spj_pos=d["spj_pos"], spj_mass=d["spj_mass"],
                   spj_quad=d["spj_quad"], epj_disp=d["epj_disp"], id_epj=d["id_epj"], spj_disp=d["spj_disp"],
                   id_spj=d["id_spj"], eps2=float(d["eps"]) ** 2, rcut2=float(d["r_out"]) ** 2,
                   G=float(d["G"]))
    return wb, d


def rel_err_vec(a: np.ndarray, ref: np.ndarray) -> np.ndarray:
    return np.linalg.norm(a - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)


def rel_err(a: np.ndarray, ref: np.ndarray) -> np.ndarray:
    return np.abs(a - ref) / np.maximum(np.abs(ref), 1e-300)


def stats(e: np.ndarray) -> dict:
    if e.size == 0:
        return dict(median=0.0, p999=0.0, max=0.0)
    return dict(median=float(np.median(e)), p999=float(np.quantile(e, 0.999)), max=float(e.max()))


def rows_batch(wb: WalkBatch, rows: np.ndarray) -> WalkBatch:
    """One walk per given EPI row, each with the lists of the row's own walk:
    the oracle on a sample of i-particles without evaluating whole walks."""
    rows = np.asarray(rows, dtype=np.int64)
    w = np.searchsorted(wb.epi_disp, rows, side="right") - 1
    ej = [wb.id_epj[wb.epj_disp[k]:wb.epj_disp[k + 1]] for k in w]
    sj = [wb.id_spj[wb.spj_disp[k]:wb.spj_disp[k + 1]] for k in w]
    disp = lambda parts: np.concatenate([[0], np.cumsum([p.size for p in parts])]).astype(np.int64)
    cat = lambda parts: np.concatenate(parts).astype(np.int32) if parts else np.zeros(0, np.int32)
    return WalkBatch(
        epi_pos=wb.epi_pos[rows], epi_rs=wb.epi_rs[rows], epi_disp=np.arange(rows.size + 1, dtype=np.int64),
        epj_pos=wb.epj_pos, epj_mass=wb.epj_mass, epj_rs=wb.epj_rs, spj_pos=wb.spj_pos, spj_mass=wb.spj_mass,
        spj_quad=wb.spj_quad, epj_disp=disp(ej), id_epj=cat(ej), spj_disp=disp(sj), id_spj=cat(sj),
        eps2=wb.eps2, rcut2=wb.rcut2, G=wb.G,
        walk_rcut2=None if wb.walk_rcut2 is None else wb.walk_rcut2[w],
        epi_index=None if wb.epi_index is None else wb.epi_index[rows])


# Mixed-precision parity bar of every GPU test: relative force and potential
# error median <= 1e-6, 99.9th percentile <= 1e-5 and max <= 1e-3 against the
# FP64 oracle, neighbour counts bit-exact.
MIXED_MEDIAN = 1e-6
MIXED_P999 = 1e-5
MIXED_MAX = 1e-3


def assert_mixed_parity(acc: np.ndarray, pot: np.ndarray, nnb: np.ndarray, o: dict, label: str = "") -> tuple:
    np.testing.assert_array_equal(nnb, o["nnb"], err_msg=f"{label} neighbour counts")
    sa, sp = stats(rel_err_vec(acc, o["acc"])), stats(rel_err(pot, o["pot"]))
    for name, s in (("force", sa), ("pot", sp)):
        assert s["median"] <= MIXED_MEDIAN and s["p999"] <= MIXED_P999 and s["max"] <= MIXED_MAX, (label, name, s)
    return sa, sp
