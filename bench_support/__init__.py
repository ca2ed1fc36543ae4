"""Support code for bench.py only (not part of the library).

``build_fp32_probe()`` compiles ``fp32_peak.cu``, the FP32 FMA throughput loops
whose measured rate is the denominator of the soft-force kernel's roofline
fraction, into ``bench_support/lib/libpgf_probe.so`` for sm_103a.

``build_fdps_driver()`` compiles ``fdps_batches.cpp``, the C++ caller that
times PeTar's unchanged multi-walk call pattern through the header functors,
into ``bench_support/lib/libpgf_fdps_batches.so``.
"""
from __future__ import annotations

import os
from pathlib import Path

HERE = Path(__file__).resolve().parent


def build_fp32_probe(force: bool = False) -> Path:
    from petar_gb300.build import ARCH_FLAGS, _newer, _nvcc, _run
    lib = HERE / "lib"
    lib.mkdir(exist_ok=True)
    out = lib / "libpgf_probe.so"
    src = HERE / "fp32_peak.cu"
    if not force and _newer(out, [src]):
        return out
    tmp = out.with_suffix(".so.tmp")
    _run([_nvcc(), *ARCH_FLAGS, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", str(src), "-o", str(tmp)])
    os.replace(tmp, out)
    return out


def build_fdps_driver(force: bool = False) -> Path:
    from petar_gb300.build import INCLUDE, _newer, _run, build_gpuforce
    lib = HERE / "lib"
    lib.mkdir(exist_ok=True)
    gf = build_gpuforce()
    out = lib / "libpgf_fdps_batches.so"
    src = HERE / "fdps_batches.cpp"
    if not force and _newer(out, [src, INCLUDE / "petar_gpuforce.hpp", INCLUDE / "petar_gpuforce.h"]):
        return out
    tmp = out.with_suffix(".so.tmp")
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", str(INCLUDE), str(src), "-o", str(tmp),
          "-L", str(gf.parent), "-lpetar_gpuforce", f"-Wl,-rpath,{gf.parent}"])
    os.replace(tmp, out)
    return out
