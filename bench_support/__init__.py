"""Support code for bench.py only (not part of the library).

``build_fp32_probe()`` compiles ``fp32_peak.cu``, the FP32 FMA throughput loops
whose measured rate is the denominator of the soft-force kernel's roofline
fraction, into ``bench_support/lib/libpgf_probe.so`` for sm_103a.
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
