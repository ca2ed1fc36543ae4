"""Generates the golden fixtures that pin the FP64 oracle to the reference.

Runs the reference's own CPU force functors -- compiled from the reference
sources by ``oracle/ref/build_ref.sh`` into ``oracle/_ref/`` -- on seeded
inputs and stores inputs and outputs as compressed ``.npz`` files next to this
script.  Needs the reference tree (only present where the fixtures are made);
the tests only read the committed ``.npz`` files.

Cases
-----
``kernel_test.npz``
    A restatement of the reference's kernel test (src/simd_test.cxx:59-131):
    1000 EPI and 2000 EPJ from an equal-mass Plummer model, 1000 random SPJ with
    the distributions of ``setSpj`` (src/simd_test.cxx:44-57), r_out = 0.01,
    eps = 1e-4, G = 1, r_search = r_out (search_factor = 0).  The RNG is this
    project's (numpy PCG64), not FDPS's.
``kernel_test_rsvar.npz``
    The same with per-particle r_search = r_out + |v| * dt * 3 (the form of
    Ptcl::calcRSearch, src/ptcl.hpp:227-238) so max(rs_i, rs_j) matters.
``plummer2048_walks.npz``
    Workload C1: Kroupa-mass Plummer sphere, N = 2048, theta = 0.3, r_out = 0.02,
    r_search = 1.5 r_out, eps = 0, lists from this package's interaction-list
    builder; reference outputs per walk.

Outputs per case and reference variant (``nosimd``: FP64 NoSimd functors;
``simd32``: AVX-512 PhantomGrapeQuad; ``simd64``: AVX-512 PhantomGrapeQuad64Bit):
EP-EP acc/pot/n_ngb and EP-SP acc/pot, G-scaled as the functors write them.

``changeover_w.npz``
    The reference's changeover functions (src/changeover.hpp, compiled into
    ``libref_changeover.so``): W_acc and W_pot of single changeovers and of
    pairs (the larger r_out wins), and the mass-scaled radii of setR(m_fac,
    r_in, r_out), on random radii with separations below r_in, inside the
    changeover, beyond r_out and on both boundaries.

``gradient_walks.npz``
    The KDKDK_4TH gradient-correction pass (src/petar.hpp:1123-1140): the
    reference's CalcCorrectEpEpWithLinearCutoffNoSimd (built with KDKDK_4TH into
    ``libref_kdkdk.so``) and its quadrupole EP-SP functor, per walk, on a
    4096-centre Plummer cluster with 30% binaries, eps = 1e-4, G = 0.9, and
    accelerations from the Plummer potential's smooth field.  Outputs: acorr
    (2 x the EP-EP sum, no G), acc (the i's own acc plus G x the SP
    acceleration) and pot (G x the SP potential), as one FDPS walk writes them.

Usage: python tests/golden/make_golden.py [fixture names]   (default: all)
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
REF_LIBS = ROOT / "oracle" / "_ref"
VARIANTS = ("nosimd", "simd32", "simd64")


def _load(variant: str):
    lib = ctypes.CDLL(str(REF_LIBS / f"libref_{variant}.so"))
    vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lib.ref_set_params.argtypes = [cd, cd, cd]
    lib.ref_epep.argtypes = [ci, vp, vp, ci, vp, vp, vp, vp, vp, vp]
    lib.ref_epsp.argtypes = [ci, vp, ci, vp, vp, vp, vp, vp]
    lib.ref_nb.argtypes = [ci, vp, vp, ci, vp, vp, vp]
    return lib


def _p(a):
    return a.ctypes.data


def run_ref(lib, eps, r_out, G, walks):
    """walks: list of dicts with xi, rsi, xj, mj, rsj, xs, ms, qs (contiguous).
    Returns per-EPI arrays concatenated in walk order."""
    lib.ref_set_params(eps, r_out, G)
    out = {k: [] for k in ("acc_ep", "pot_ep", "nnb_ep", "acc_sp", "pot_sp", "nnb_search")}
    for w in walks:
        ni, nj, ns = w["rsi"].size, w["mj"].size, w["ms"].size
        a = np.zeros((ni, 3)); p = np.zeros(ni); n = np.zeros(ni, np.int64)
        lib.ref_epep(ni, _p(w["xi"]), _p(w["rsi"]), nj, _p(w["xj"]), _p(w["mj"]), _p(w["rsj"]),
                     _p(a), _p(p), _p(n))
        out["acc_ep"].append(a); out["pot_ep"].append(p); out["nnb_ep"].append(n)
        a = np.zeros((ni, 3)); p = np.zeros(ni)
        if ns:
            lib.ref_epsp(ni, _p(w["xi"]), ns, _p(w["xs"]), _p(w["ms"]), _p(w["qs"]), _p(a), _p(p))
        out["acc_sp"].append(a); out["pot_sp"].append(p)
        n = np.zeros(ni, np.int64)
        lib.ref_nb(ni, _p(w["xi"]), _p(w["rsi"]), nj, _p(w["xj"]), _p(w["rsj"]), _p(n))
        out["nnb_search"].append(n)
    return {k: np.concatenate(v) for k, v in out.items()}


def kernel_test_case(seed: int, rs_var: bool) -> dict:
    from petar_gb300 import ics
    rng = np.random.default_rng(seed)
    n_epi, n_epj, n_spj = 1000, 2000, 1000
    N = max(n_epi, n_epj)
    mass = np.full(N, 1.0 / N)
    pos, vel = ics.plummer(rng, mass)
    r_out, eps, G = 0.01, 1e-4, 1.0
    if rs_var:
        rs = r_out + np.sqrt((vel ** 2).sum(1)) * (1.0 / 2048.0) * 3.0
    else:
        rs = np.full(N, r_out)
    # setSpj (src/simd_test.cxx:44-57): mass 1/N + 0.001/N * U, pos 1 + 10 U, quad 10 U.
    sm = 1.0 / N + 0.001 / N * rng.random(n_spj)
    sp = 1.0 + 10.0 * rng.random((n_spj, 3))
    q = 10.0 * rng.random((n_spj, 6))
    return dict(epi_pos=pos[:n_epi].copy(), epi_rs=rs[:n_epi].copy(), epj_pos=pos[:n_epj].copy(),
                epj_mass=mass[:n_epj].copy(), epj_rs=rs[:n_epj].copy(), spj_pos=sp, spj_mass=sm,
                spj_quad=q, epi_disp=np.array([0, n_epi], np.int64),
                epj_disp=np.array([0, n_epj], np.int64), id_epj=np.arange(n_epj, dtype=np.int32),
                spj_disp=np.array([0, n_spj], np.int64), id_spj=np.arange(n_spj, dtype=np.int32),
                eps=np.float64(eps), r_out=np.float64(r_out), G=np.float64(G))


def plummer2048_case(seed: int) -> dict:
    from petar_gb300 import ics, walks
    cl = ics.make_plummer_cluster(seed, 2048, 0.02, binary_fraction=0.0, theta=0.3, n_group_limit=512)
    wb = walks.build_walks(cl)
    return dict(epi_pos=wb.epi_pos, epi_rs=wb.epi_rs, epj_pos=wb.epj_pos, epj_mass=wb.epj_mass,
                epj_rs=wb.epj_rs, spj_pos=wb.spj_pos, spj_mass=wb.spj_mass, spj_quad=wb.spj_quad,
                epi_disp=wb.epi_disp, epj_disp=wb.epj_disp, id_epj=wb.id_epj, spj_disp=wb.spj_disp,
                id_spj=wb.id_spj, eps=np.float64(0.0), r_out=np.float64(cl.r_out), G=np.float64(1.0))


def walks_of(case: dict) -> list[dict]:
    out = []
    nw = case["epi_disp"].size - 1
    for w in range(nw):
        i0, i1 = case["epi_disp"][w], case["epi_disp"][w + 1]
        je = case["id_epj"][case["epj_disp"][w]:case["epj_disp"][w + 1]]
        js = case["id_spj"][case["spj_disp"][w]:case["spj_disp"][w + 1]]
        c = np.ascontiguousarray
        out.append(dict(xi=c(case["epi_pos"][i0:i1]), rsi=c(case["epi_rs"][i0:i1]),
                        xj=c(case["epj_pos"][je]), mj=c(case["epj_mass"][je]), rsj=c(case["epj_rs"][je]),
                        xs=c(case["spj_pos"][js]), ms=c(case["spj_mass"][js]), qs=c(case["spj_quad"][js])))
    return out


def changeover_case(seed: int) -> dict:
    """Inputs and reference outputs of the changeover W functions."""
    lib = ctypes.CDLL(str(REF_LIBS / "libref_changeover.so"))
    vp, ci = ctypes.c_void_p, ctypes.c_int
    lib.ref_co_w.argtypes = [ci] + [vp] * 5
    lib.ref_co_w_two.argtypes = [ci] + [vp] * 7
    lib.ref_co_setr_mfac.argtypes = [ci] + [vp] * 5
    rng = np.random.default_rng(seed)
    n = 6000
    r_out = 10 ** rng.uniform(-4, -1, n)
    r_in = r_out * rng.uniform(0.05, 0.5, n)
    u = rng.uniform(-0.3, 1.3, n)
    dr = r_in + u * (r_out - r_in)
    dr[:200] = r_in[:200]
    dr[200:400] = r_out[200:400]
    dr[400:600] = rng.uniform(0, 1, 200) * r_in[400:600]
    dr = np.abs(dr)
    acc0w = np.zeros(n)
    potw = np.zeros(n)
    lib.ref_co_w(n, _p(r_in), _p(r_out), _p(dr), _p(acc0w), _p(potw))
    r_out2 = r_out * rng.uniform(0.5, 2.0, n)
    r_out2[:300] = r_out[:300]  # ties: the second changeover wins
    r_in2 = r_out2 * rng.uniform(0.05, 0.5, n)
    acc0w2 = np.zeros(n)
    potw2 = np.zeros(n)
    lib.ref_co_w_two(n, _p(r_in), _p(r_out), _p(r_in2), _p(r_out2), _p(dr), _p(acc0w2), _p(potw2))
    m_fac = 10 ** rng.uniform(-2, 2.5, n)
    rin_m = np.zeros(n)
    rout_m = np.zeros(n)
    lib.ref_co_setr_mfac(n, _p(m_fac), _p(r_in), _p(r_out), _p(rin_m), _p(rout_m))
    return dict(r_in=r_in, r_out=r_out, dr=dr, acc0w=acc0w, potw=potw, r_in2=r_in2, r_out2=r_out2,
                acc0w_two=acc0w2, potw_two=potw2, m_fac=m_fac, r_in_mfac=rin_m, r_out_mfac=rout_m)


def gradient_case(seed: int) -> dict:
    """Walks and accelerations for the gradient-correction fixture."""
    from petar_gb300 import ics, walks
    cl = ics.make_plummer_cluster(seed, 4096, 0.015, binary_fraction=0.3, theta=0.3)
    wb = walks.build_walks(cl)
    b2 = (3.0 * np.pi / 16.0) ** 2  # Plummer scale length squared in Henon units
    acc = -wb.epj_pos / ((wb.epj_pos ** 2).sum(1) + b2)[:, None] ** 1.5
    return dict(epi_pos=wb.epi_pos, epi_rs=wb.epi_rs, epj_pos=wb.epj_pos, epj_mass=wb.epj_mass,
                epj_rs=wb.epj_rs, spj_pos=wb.spj_pos, spj_mass=wb.spj_mass, spj_quad=wb.spj_quad,
                epi_disp=wb.epi_disp, epj_disp=wb.epj_disp, id_epj=wb.id_epj, spj_disp=wb.spj_disp,
                id_spj=wb.id_spj, eps=np.float64(1e-4), r_out=np.float64(cl.r_out), G=np.float64(0.9),
                epi_acc=acc.copy(), epj_acc=acc.copy())


def run_ref_gradient(case: dict) -> dict:
    lib = _load("kdkdk")
    vp, ci = ctypes.c_void_p, ctypes.c_int
    lib.ref_correct.argtypes = [ci, vp, vp, ci, vp, vp, vp, vp, vp]
    lib.ref_set_params(float(case["eps"]), float(case["r_out"]), float(case["G"]))
    c = np.ascontiguousarray
    out = {k: [] for k in ("acorr", "acc", "pot")}
    for w in range(case["epi_disp"].size - 1):
        i0, i1 = case["epi_disp"][w], case["epi_disp"][w + 1]
        je = case["id_epj"][case["epj_disp"][w]:case["epj_disp"][w + 1]]
        js = case["id_spj"][case["spj_disp"][w]:case["spj_disp"][w + 1]]
        xi, ai = c(case["epi_pos"][i0:i1]), c(case["epi_acc"][i0:i1])
        xj, mj, aj = c(case["epj_pos"][je]), c(case["epj_mass"][je]), c(case["epj_acc"][je])
        ni = i1 - i0
        acorr = np.zeros((ni, 3)); acc_i = np.zeros((ni, 3))
        lib.ref_correct(ni, _p(xi), _p(ai), je.size, _p(xj), _p(mj), _p(aj), _p(acorr), _p(acc_i))
        a_sp = np.zeros((ni, 3)); p_sp = np.zeros(ni)
        if js.size:
            # keep the gathered arrays referenced while the C call reads them
            xs, ms, qs = c(case["spj_pos"][js]), c(case["spj_mass"][js]), c(case["spj_quad"][js])
            lib.ref_epsp(ni, _p(xi), js.size, _p(xs), _p(ms), _p(qs), _p(a_sp), _p(p_sp))
        out["acorr"].append(acorr); out["acc"].append(acc_i + a_sp); out["pot"].append(p_sp)
    return {k: np.concatenate(v) for k, v in out.items()}


def main() -> None:
    if not (REF_LIBS / "libref_nosimd.so").exists() or not (REF_LIBS / "libref_changeover.so").exists():
        # The reference checkout: PETAR_REFERENCE_ROOT, else the one this project was built against.
        ref = os.environ.get("PETAR_REFERENCE_ROOT", "/root/reference")
        subprocess.run([str(ROOT / "oracle" / "ref" / "build_ref.sh"), ref], check=True)
    sys.path.insert(0, str(ROOT))
    only = set(sys.argv[1:])
    if not only or "changeover_w" in only:
        np.savez_compressed(HERE / "changeover_w.npz", **changeover_case(77))
        print("changeover_w")
    if not only or "gradient_walks" in only:
        case = gradient_case(12)
        payload = dict(case)
        payload.update({f"ref__{k}": v for k, v in run_ref_gradient(case).items()})
        np.savez_compressed(HERE / "gradient_walks.npz", **payload)
        print("gradient_walks")
    if only and not only - {"changeover_w", "gradient_walks"}:
        return
    cases = {
        "kernel_test": kernel_test_case(20240, rs_var=False),
        "kernel_test_rsvar": kernel_test_case(20241, rs_var=True),
        "plummer2048_walks": plummer2048_case(1),
    }
    libs = {v: _load(v) for v in VARIANTS if (REF_LIBS / f"libref_{v}.so").exists()}
    for name, case in cases.items():
        if only and name not in only:
            continue
        ws = walks_of(case)
        payload = dict(case)
        for v, lib in libs.items():
            res = run_ref(lib, float(case["eps"]), float(case["r_out"]), float(case["G"]), ws)
            for k, a in res.items():
                payload[f"{v}__{k}"] = a
        np.savez_compressed(HERE / f"{name}.npz", **payload)
        print(name, {k: v.shape for k, v in payload.items() if "__" in k and k.endswith("nnb_ep")})


if __name__ == "__main__":
    main()
