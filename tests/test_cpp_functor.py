"""The header-only C++ functors (include/petar_gpuforce.hpp) compile against
PeTar-layout record types and, driven in FDPS's call order, reproduce the
oracle."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from helpers import assert_mixed_parity, load_golden
from petar_gb300.build import build_gpuforce

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "functor_test.cpp"


def compile_driver(tmp_path: Path) -> Path:
    lib = build_gpuforce()
    exe = tmp_path / "functor_test"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(SRC), "-o", str(exe),
                    "-L", str(lib.parent), "-lpetar_gpuforce", f"-Wl,-rpath,{lib.parent}"], check=True)
    return exe


def test_functor_header_compiles(tmp_path):
    assert compile_driver(tmp_path).exists()


def write_case(wb, path: Path) -> None:
    with open(path, "wb") as f:
        np.array([wb.n_walk, wb.epj_mass.size, wb.spj_mass.size, wb.epi_rs.size, wb.id_epj.size,
                  wb.id_spj.size], np.int64).tofile(f)
        np.array([wb.eps2, wb.rcut2, wb.G], np.float64).tofile(f)
        for a in (wb.n_epi, wb.n_epj, wb.n_spj):
            np.asarray(a, np.int32).tofile(f)
        for a in (wb.epi_pos, wb.epi_rs, wb.epj_mass, wb.epj_pos, wb.epj_rs, wb.spj_mass, wb.spj_pos,
                  wb.spj_quad):
            np.ascontiguousarray(a, np.float64).tofile(f)
        for a in (wb.id_epj, wb.id_spj):
            np.asarray(a, np.int32).tofile(f)


@pytest.mark.gpu
def test_functor_matches_oracle(tmp_path):
    exe = compile_driver(tmp_path)
    wb, _ = load_golden("plummer2048_walks")
    write_case(wb, tmp_path / "in.bin")
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True)
    ni = wb.epi_rs.size
    raw = np.fromfile(tmp_path / "out.bin", np.uint8)
    acc = raw[:24 * ni].view(np.float64).reshape(ni, 3)
    pot = raw[24 * ni:32 * ni].view(np.float64)
    nnb = raw[32 * ni:40 * ni].view(np.int64)
    # The drop-in path PeTar calls: the full mixed-precision bar (median,
    # 99.9th percentile and max relative error, counts exact).
    assert_mixed_parity(acc, pot, nnb, oracle.force(wb), label="C++ functor")


NBODY_SRC = ROOT / "tests" / "cpp" / "nbody_test.cpp"


def compile_nbody_driver(tmp_path: Path) -> Path:
    lib = build_gpuforce()
    exe = tmp_path / "nbody_test"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(NBODY_SRC), "-o", str(exe),
                    "-L", str(lib.parent), "-lpetar_gpuforce", f"-Wl,-rpath,{lib.parent}"], check=True)
    return exe


def test_nbody_wrapper_compiles(tmp_path):
    assert compile_nbody_driver(tmp_path).exists()


@pytest.mark.gpu
def test_nbody_wrapper_matches_python_binding(tmp_path):
    """The C++ DeviceTreeStep and the Python binding run the same steps on
    the same library: results agree bit for bit."""
    from petar_gb300 import ics, nbody
    exe = compile_nbody_driver(tmp_path)
    cl = ics.make_plummer_cluster(8, 8192, 0.01, binary_fraction=0.2)
    steps, dt = 4, 1.0 / 1024
    with open(tmp_path / "in.bin", "wb") as f:
        np.array([cl.n, steps], np.int64).tofile(f)
        np.array([dt, cl.eps ** 2, cl.r_out, cl.G, cl.theta], np.float64).tofile(f)
        np.array([cl.n_leaf_limit, cl.n_group_limit], np.int32).tofile(f)
        for a in (cl.pos, cl.vel, cl.mass, cl.r_search):
            np.ascontiguousarray(a, np.float64).tofile(f)
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True)
    n = cl.n
    raw = np.fromfile(tmp_path / "out.bin", np.uint8)
    pos = raw[:24 * n].view(np.float64).reshape(n, 3)
    acc = raw[24 * n:48 * n].view(np.float64).reshape(n, 3)
    pot = raw[48 * n:56 * n].view(np.float64)
    nnb = raw[56 * n:60 * n].view(np.int32)
    with nbody.DeviceNBody(cl) as h:
        h.run(steps, dt, graph=True)
        st = h.state()
    np.testing.assert_array_equal(pos, st["pos"])
    np.testing.assert_array_equal(acc, st["acc"])
    np.testing.assert_array_equal(pot, st["pot"])
    np.testing.assert_array_equal(nnb, st["n_ngb"])
