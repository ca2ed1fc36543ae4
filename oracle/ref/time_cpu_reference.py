"""Times the reference's own CPU force paths on an x86 host over the bench
workload's lists, and writes the summary that bench.py reports as its
``cpu_reference_x86`` side record.

The reference's default CPU path is the AVX-512 PhantomGrapeQuad kernel
(src/phantomquad_for_p3t_x86.hpp, FP32 with one Newton-Raphson step for EP-EP,
``-DRSQRT_NR_EPJ_X2``), its 64-bit build (P3T_64BIT) the PhantomGrapeQuad64Bit
kernel, and the FP64 NoSimd functors (src/soft_force.hpp) the portable one.
All three are x86 code compiled from the reference sources by build_ref.sh;
the GPU hosts are aarch64, so the measurement runs here and is committed.

Workload: Plummer, 1,048,576 centres of mass with 50% binaries (1,572,864
particles), theta 0.3, r_out 0.003 (bench.py's plummer1m_bin50), on the same
seeded half of the walks that bench.py's CPU legs time (seed 7).  Each library
runs every sampled walk with OpenMP over walks on all host threads
(ref_force_walks in ref_driver.cpp).  Accuracy is stated against the NoSimd
functors, which the oracle reproduces bit for bit.

Usage (from the repository root, after build_ref.sh):
    python oracle/ref/time_cpu_reference.py [output.md]
"""
from __future__ import annotations

import ctypes
import json
import os
import platform
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from petar_gb300 import ics, walks  # noqa: E402

REF = ROOT / "oracle" / "_ref"
SAMPLE_FRACTION, SAMPLE_SEED = 0.5, 7


def run(lib_path: Path, b) -> tuple[float, dict]:
    lib = ctypes.CDLL(str(lib_path))
    vp = ctypes.c_void_p
    lib.ref_set_params.argtypes = [ctypes.c_double] * 3
    lib.ref_force_walks.argtypes = [ctypes.c_int] + [vp] * 16
    lib.ref_set_params(float(np.sqrt(b.eps2)), float(np.sqrt(b.rcut2)), float(b.G))
    c = lambda a, t: np.ascontiguousarray(a, dtype=t)
    arrs = [c(b.epi_disp, np.int64), c(b.epi_pos, np.float64), c(b.epi_rs, np.float64),
            c(b.epj_disp, np.int64), c(b.id_epj, np.int32), c(b.spj_disp, np.int64), c(b.id_spj, np.int32),
            c(b.epj_pos, np.float64), c(b.epj_mass, np.float64), c(b.epj_rs, np.float64),
            c(b.spj_pos, np.float64), c(b.spj_mass, np.float64), c(b.spj_quad, np.float64)]
    ni = b.epi_rs.size
    out = dict(acc=np.zeros((ni, 3)), pot=np.zeros(ni), nnb=np.zeros(ni, np.int64))
    args = [b.n_walk] + [a.ctypes.data for a in arrs] + [out["acc"].ctypes.data, out["pot"].ctypes.data,
                                                        out["nnb"].ctypes.data]
    lib.ref_force_walks(*args)  # warm-up (first-touch of the per-thread buffers)
    t = time.time()
    lib.ref_force_walks(*args)
    return time.time() - t, out


def main() -> None:
    out_path = Path(sys.argv[1]) if len(sys.argv) > 1 else ROOT / "profiles" / "cpu_reference_x86_plummer1m_bin50.md"
    cl = ics.make_plummer_cluster(3, 1048576, 0.003, binary_fraction=0.5, theta=0.3)
    wb = walks.build_walks(cl)
    order = np.random.default_rng(SAMPLE_SEED).permutation(wb.n_walk)
    sw = np.sort(order[:max(1, int(round(SAMPLE_FRACTION * wb.n_walk)))])
    b = wb.subset(sw)
    n_int = int(sum(b.interactions()))
    cpu = platform.processor() or platform.machine()
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.startswith("model name"):
                cpu = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    rec = {"workload": "plummer1m_bin50", "host": cpu, "cores": os.cpu_count(),
           "sample": f"{b.n_walk} of {wb.n_walk} walks chosen at random (seed {SAMPLE_SEED}), {n_int:.3e} "
                     f"interactions", "unit": "Ginteractions/s", "kernels": {}}
    ref64 = None
    for key, name in (("nosimd_fp64", "libref_nosimd.so"), ("avx512_fp32", "libref_simd32.so"),
                      ("avx512_64bit", "libref_simd64.so")):
        p = REF / name
        if not p.exists():
            continue
        dt, res = run(p, b)
        entry = {"seconds": dt, "value": n_int / dt / 1e9}
        if key == "nosimd_fp64":
            ref64 = res
        elif ref64 is not None:
            ea = np.linalg.norm(res["acc"] - ref64["acc"], axis=1) / np.linalg.norm(ref64["acc"], axis=1)
            ep = np.abs(res["pot"] - ref64["pot"]) / np.abs(ref64["pot"])
            entry["accuracy_vs_fp64"] = {"force_rel_err_median": float(np.median(ea)),
                                         "force_rel_err_p999": float(np.quantile(ea, 0.999)),
                                         "force_rel_err_max": float(ea.max()),
                                         "pot_rel_err_p999": float(np.quantile(ep, 0.999)),
                                         "n_ngb_mismatches": int((res["nnb"] != ref64["nnb"]).sum())}
        rec["kernels"][key] = entry
        print(key, entry, flush=True)
    lines = [
        "# Reference CPU force paths on x86 (AVX-512), Plummer 1M binary workload",
        "",
        "The reference's own CPU kernels, compiled from its sources by `oracle/ref/build_ref.sh`, timed over",
        "the same seeded half of the walks that `bench.py`'s CPU legs use, with OpenMP over walks on every",
        "host thread. The GPU hosts are aarch64, so this x86 measurement is a side record with its own host",
        f"and core count: {cpu}, {os.cpu_count()} threads.",
        "",
        "Command: `python oracle/ref/time_cpu_reference.py` (after `bash oracle/ref/build_ref.sh <PeTar checkout>`).",
        "",
        "| Kernel | Seconds | Ginteractions/s | force p99.9 / max vs FP64 | count mismatches |",
        "|---|---|---|---|---|",
    ]
    for k, e in rec["kernels"].items():
        a = e.get("accuracy_vs_fp64")
        acc = f"{a['force_rel_err_p999']:.2e} / {a['force_rel_err_max']:.2e}" if a else "(the FP64 reference)"
        cnt = str(a["n_ngb_mismatches"]) if a else "0"
        lines.append(f"| {k} | {e['seconds']:.2f} | {e['value']:.3f} | {acc} | {cnt} |")
    lines += ["", "record: " + json.dumps(rec), ""]
    out_path.write_text("\n".join(lines))
    print("wrote", out_path)


if __name__ == "__main__":
    main()
