"""Builds the native parts of petar_gb300 in-tree.

Products (all under ``petar_gb300/lib``):

* ``libpetar_gpuforce.so`` -- the soft-force kernels for sm_103a and the C ABI
  declared in ``include/petar_gpuforce.h``.
* ``libpgf_harness.so``   -- the host-side interaction-list builder that plays
  FDPS's role for tests and benchmarks.

Everything is compiled with plain ``nvcc`` / ``g++`` command lines, in
parallel, with one ``-gencode`` (sm_103a).  Nothing here is x86-specific, so the
same recipe runs on the aarch64 GPU hosts.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB = PKG / "lib"
INCLUDE = ROOT / "include"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the soft-force kernels need the CUDA toolkit")


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def _newer(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(s.stat().st_mtime <= t for s in sources)


GPU_SOURCES = [
    "gpuforce/pgf_api.cu",
    "gpuforce/pgf_kernels_fp64.cu",
    "gpuforce/pgf_kernels_mixed.cu",
    "gpuforce/pgf_kernels_ws.cu",
    "gpuforce/pgf_noalloc.cu",
    "gpuforce/pgf_hostdirect.cu",
    "gpuforce/pgf_kernels_gradient.cu",
    "gpuforce/pgf_nbody.cu",
]
# Per-file flags: the device list builder repeats the host builder's FP64
# arithmetic exactly, so nothing in it may be contracted into an FMA.
GPU_FILE_FLAGS = {
    "pgf_nbody": ["-fmad=false"],
}
GPU_HEADERS = [
    "gpuforce/pgf_internal.cuh",
]


def build_gpuforce(force: bool = False, verbose: bool = False) -> Path:
    """Compiles the kernels + C ABI into ``lib/libpetar_gpuforce.so``."""
    LIB.mkdir(exist_ok=True)
    out = LIB / "libpetar_gpuforce.so"
    srcs = [CSRC / s for s in GPU_SOURCES]
    deps = srcs + [CSRC / h for h in GPU_HEADERS] + [INCLUDE / "petar_gpuforce.h"]
    if not force and _newer(out, deps):
        return out
    nvcc = _nvcc()
    objdir = LIB / "obj"
    objdir.mkdir(exist_ok=True)
    # Host code without FP contraction: the host packing and the host-direct
    # gather kernels must round every FP64 operation the same way.
    common = [nvcc, *ARCH_FLAGS, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fopenmp", "-Xcompiler", "-ffp-contract=off", "-I", str(INCLUDE),
              "-I", str(CSRC / "gpuforce")]
    if verbose:
        common += ["-Xptxas", "-v"]

    def compile_one(src: Path) -> Path:
        obj = objdir / (src.stem + ".o")
        _run(common + GPU_FILE_FLAGS.get(src.stem, []) + ["-c", str(src), "-o", str(obj)])
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = out.with_suffix(".so.tmp")
    _run([nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs),
          "-Xcompiler", "-fopenmp", "-lcuda", "-lgomp"])
    os.replace(tmp, out)
    return out


def build_harness(force: bool = False) -> Path:
    """Compiles the interaction-list builder into ``lib/libpgf_harness.so``."""
    LIB.mkdir(exist_ok=True)
    out = LIB / "libpgf_harness.so"
    src = CSRC / "harness" / "walk_builder.cpp"
    if not force and _newer(out, [src]):
        return out
    tmp = out.with_suffix(".so.tmp")
    # No FMA contraction: the device list builder reproduces its FP64 results bit for bit.
    _run(["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp", str(src), "-o", str(tmp)])
    os.replace(tmp, out)
    return out


def build_all(force: bool = False, verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        futs = [ex.submit(build_gpuforce, force, verbose), ex.submit(build_harness, force)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose="-v" in sys.argv)
