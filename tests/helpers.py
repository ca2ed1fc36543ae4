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
