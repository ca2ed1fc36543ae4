#!/usr/bin/env python
"""Soft-force benchmark: tree-force Ginteractions/s at N = 1M.

Workload (default ``plummer1m_bin50``): Plummer sphere of 1,048,576 centres of
mass with 50% primordial binaries (1,572,864 particles), Kroupa IMF, Henon
units, theta = 0.3, quadrupole superparticles, n_leaf_limit 20,
n_group_limit 512, r_out = 0.003, r_in = 0.1 r_out, r_search = 1.5 r_out,
eps = 0.  Interaction lists come from the package's interaction-list builder
(the FDPS stand-in).  One step = one multi-walk force evaluation over all
walks.

Reported (one JSON line from rank 0):
* value: Ginteractions/s of the mixed-precision kernels on device-resident
  lists (sum over ranks / max rank time), with the L2 flushed between steps;
* fp64_plain: the same for the plain FP64 kernel, and the speed-up;
* accuracy: mixed vs FP64 kernel on every particle (relative force and
  potential error; neighbour-count mismatches);
* e2e: the same metric through the C ABI with host records (pack, copies,
  kernels, copy back, unpack) per step;
* roofline: FP32 flops (19 per EP-EP, 54 per EP-SP interaction) of the main
  kernel per launch over its event-timed duration, against an FP32 FMA peak
  measured in the same run;
* cpu_baseline: the FP64 oracle (a CPU port of the reference functors) on a
  sample of the walks, with every host thread;
* modes: neighbour search, fused changeover and KDKDK_4TH gradient passes on
  the same lists;
* configs: the bench workload through the functors in PeTar's unchanged
  batches of 200 walks per call; Plummer N = 65,536 (mixed against the plain FP64 kernel) and the
  64-cluster ensemble in one launch (against 64 sequential plain FP64
  launches), each timed on its own resident lists;
* kdk_graph: the King W0 = 7, N = 4,194,304 configuration (theta 0.4,
  r_out 0.0015) run device-resident: tree, lists, force, kicks and drifts of
  100 leapfrog steps of dt = 1/1024 in one CUDA graph.

``--impl reference`` times the reference's own CPU path instead (the
reference functors compiled from its sources when they are present on this
host, else the oracle port) and prints the same metric with impl=reference.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    "plummer1m_bin50": dict(seed=3, n_cm=1048576, r_out=0.003, binary_fraction=0.5, theta=0.3),
    "plummer256k_bin50": dict(seed=4, n_cm=262144, r_out=0.0048, binary_fraction=0.5, theta=0.3),
    "plummer65k": dict(seed=2, n_cm=65536, r_out=0.008, binary_fraction=0.0, theta=0.3),
    "plummer2k": dict(seed=1, n_cm=2048, r_out=0.02, binary_fraction=0.0, theta=0.3),
}
FLOPS_EPEP = 19
FLOPS_EPSP = 54


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """Largest value of x over all ranks (the step time that bounds the job)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(interactions_per_rank: int, steps: int, t_max_s: float, world: int) -> float:
    """Whole-job Ginteractions/s: every rank evaluates its own replica, so the
    job does world x interactions per step in the slowest rank's time."""
    return world * interactions_per_rank * steps / t_max_s / 1e9


def make_workload(name: str, rank: int):
    from petar_gb300 import ics, walks
    w = WORKLOADS[name]
    t = time.time()
    cl = ics.make_plummer_cluster(w["seed"] + 1000 * rank, w["n_cm"], w["r_out"],
                                  binary_fraction=w["binary_fraction"], theta=w["theta"])
    wb = walks.build_walks(cl)
    log(f"[rank {rank}] workload {name}: {cl.n} particles, {wb.n_walk} walks, built in {time.time() - t:.1f}s")
    return cl, wb


class NvmlSampler:
    """SM clock and clock-event reasons every 2 ms through NVML (ctypes), in a
    background thread, while running."""
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, pci_bus_id: str | None, index: int):
        import ctypes
        import threading
        self.ok = False
        self.samples, self.reasons, self.max_mhz = [], set(), None
        try:
            self.nvml = ctypes.CDLL("libnvidia-ml.so.1")
            if self.nvml.nvmlInit_v2() != 0:
                return
            self.h = ctypes.c_void_p()
            rc = 1
            if pci_bus_id:
                rc = self.nvml.nvmlDeviceGetHandleByPciBusId_v2(pci_bus_id.encode(), ctypes.byref(self.h))
            if rc != 0:
                rc = self.nvml.nvmlDeviceGetHandleByIndex_v2(index, ctypes.byref(self.h))
            if rc != 0:
                return
            mx = ctypes.c_uint()
            if self.nvml.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(mx)) == 0:
                self.max_mhz = mx.value
            self.reason_fn = getattr(self.nvml, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                getattr(self.nvml, "nvmlDeviceGetCurrentClocksThrottleReasons", None)
            self.ok = True
        except (OSError, AttributeError):
            return
        self._stop = threading.Event()
        self._thread = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        import ctypes
        clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
        while not self._stop.is_set():
            if self.nvml.nvmlDeviceGetClockInfo(self.h, 1, ctypes.byref(clk)) == 0:
                self.samples.append(clk.value)
            if self.reason_fn is not None and self.reason_fn(self.h, ctypes.byref(rs)) == 0:
                for bit, name in self.REASONS.items():
                    if rs.value & bit:
                        self.reasons.add(name)
            time.sleep(0.002)

    def __enter__(self):
        if self.ok:
            self._thread.start()
        return self

    def __exit__(self, *exc):
        if self.ok:
            self._stop.set()
            self._thread.join()

    def summary(self) -> dict | None:
        if not self.ok or not self.samples:
            return None
        return {"sm_mhz": statistics.median(self.samples), "sm_max_mhz": self.max_mhz,
                "reasons": sorted(self.reasons), "samples": len(self.samples), "source": "nvml"}


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = [l.split(",") for l in Path(self.file.name).read_text().splitlines() if l.strip()]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        os.unlink(self.file.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp32_peak_tflops() -> dict:
    """FP32 FMA throughput of this GPU, measured with scalar FMAs and with
    packed FP32x2 FMAs (TFLOP/s, best of three)."""
    import ctypes
    from bench_support import build_fp32_probe
    lib = ctypes.CDLL(str(build_fp32_probe()))
    out = {}
    for key, fn in (("ffma", lib.pgf_probe_fp32_peak), ("ffma2", lib.pgf_probe_fp32x2_peak)):
        fn.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        best = None
        for _ in range(3):
            tf, ms = ctypes.c_double(), ctypes.c_double()
            if fn(20000, ctypes.byref(tf), ctypes.byref(ms)) == 0:
                best = tf.value if best is None else max(best, tf.value)
        out[key] = best
    return out


def traffic_from_profiles() -> float | None:
    """DRAM bytes per launch of the main kernel from the committed ncu summary
    (a line 'dram_bytes_per_launch_scaled: <bytes>'), or None."""
    # A capture of the 1M workload itself, else a smaller capture scaled to it.
    for name, key in (("ws_kernel_plummer1m_bin50.md", "dram_bytes_per_launch"),
                      ("ws_kernel_plummer256k_bin50.md", "dram_bytes_per_launch_scaled")):
        p = ROOT / "profiles" / name
        if p.exists():
            m = re.search(key + r":\s*([0-9.eE+]+)", p.read_text())
            if m:
                return float(m.group(1))
    return None


def accuracy_violations(acc: dict) -> list[str]:
    """Mixed-precision results against the plain FP64 kernel on every particle
    of the workload: median <= 1e-6, 99.9th percentile <= 1e-5 and max <= 1e-3
    relative error for force and potential, neighbour counts equal."""
    bad = []
    for q in ("force", "pot"):
        for stat, bound in (("median", 1e-6), ("p999", 1e-5), ("max", 1e-3)):
            v = acc[f"{q}_rel_err_{stat}"]
            if not v <= bound:
                bad.append(f"{q} {stat} {v:.3g} > {bound:g}")
    if acc["n_ngb_mismatches"]:
        bad.append(f"{acc['n_ngb_mismatches']} neighbour-count mismatches")
    return bad


CPU_SAMPLE_FRACTION = 0.5  # of the walks, seeded: the same sample in both legs
CPU_SAMPLE_SEED = 7


def sample_walks(wb, fraction: float = CPU_SAMPLE_FRACTION, seed: int = CPU_SAMPLE_SEED) -> np.ndarray:
    """The CPU legs' sample: a seeded random fraction of the walks (the same
    walks in the GPU arm's cpu_baseline and in --impl reference)."""
    order = np.random.default_rng(seed).permutation(wb.n_walk)
    k = max(1, int(round(fraction * wb.n_walk)))
    return np.sort(order[:k])


def cpu_reference_runner():
    """The reference's own FP64 functors when compiled on this host
    (oracle/_ref), else the oracle port.  Returns (kind, run(batch))."""
    import ctypes
    from concurrent.futures import ThreadPoolExecutor
    import oracle
    ref = ROOT / "oracle" / "_ref" / "libref_nosimd.so"
    lib = None
    if ref.exists():
        try:
            lib = ctypes.CDLL(str(ref))
        except OSError:
            lib = None
    if lib is None:
        return "port", lambda b: oracle.force(b)
    vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lib.ref_set_params.argtypes = [cd, cd, cd]
    lib.ref_epep.argtypes = [ci, vp, vp, ci, vp, vp, vp, vp, vp, vp]
    lib.ref_epsp.argtypes = [ci, vp, ci, vp, vp, vp, vp, vp]

    def run(b):
        lib.ref_set_params(float(np.sqrt(b.eps2)), float(np.sqrt(b.rcut2)), float(b.G))

        def one(w):
            i0, i1 = b.epi_disp[w], b.epi_disp[w + 1]
            ni = int(i1 - i0)
            je = b.id_epj[b.epj_disp[w]:b.epj_disp[w + 1]]
            js = b.id_spj[b.spj_disp[w]:b.spj_disp[w + 1]]
            xi = np.ascontiguousarray(b.epi_pos[i0:i1])
            rsi = np.ascontiguousarray(b.epi_rs[i0:i1])
            xj, mj, rsj = (np.ascontiguousarray(a[je]) for a in (b.epj_pos, b.epj_mass, b.epj_rs))
            xs, ms, qs = (np.ascontiguousarray(a[js]) for a in (b.spj_pos, b.spj_mass, b.spj_quad))
            a = np.zeros((ni, 3)); p = np.zeros(ni); n = np.zeros(ni, np.int64)
            lib.ref_epep(ni, xi.ctypes.data, rsi.ctypes.data, je.size, xj.ctypes.data, mj.ctypes.data,
                         rsj.ctypes.data, a.ctypes.data, p.ctypes.data, n.ctypes.data)
            a2 = np.zeros((ni, 3)); p2 = np.zeros(ni)
            if js.size:
                lib.ref_epsp(ni, xi.ctypes.data, js.size, xs.ctypes.data, ms.ctypes.data, qs.ctypes.data,
                             a2.ctypes.data, p2.ctypes.data)
            return a + a2

        with ThreadPoolExecutor(max_workers=os.cpu_count()) as ex:
            list(ex.map(one, range(b.n_walk)))

    return "reference", run


def time_cpu(wb) -> tuple[str, dict, callable]:
    """The CPU legs' runner and their fixed seeded sample of the walks."""
    kind, run = cpu_reference_runner()
    sub = wb.subset(sample_walks(wb))
    n_int = sum(sub.interactions())
    desc = (f"{sub.n_walk} of {wb.n_walk} walks chosen at random (seed {CPU_SAMPLE_SEED}), {n_int:.3e} of "
            f"{sum(wb.interactions()):.3e} interactions")
    return kind, dict(batch=sub, n_int=n_int, desc=desc), run


def workload_config(name: str, cl, wb) -> dict:
    """The `config` of both arms' JSON lines."""
    n_epep, n_epsp = wb.interactions()
    return {"workload": name, "n_particles": int(cl.n), "n_walk": int(wb.n_walk),
            "interactions_epep": int(n_epep), "interactions_epsp": int(n_epsp),
            "theta": WORKLOADS[name]["theta"], "r_out": WORKLOADS[name]["r_out"],
            "l2": "flushed between steps (256 MB write)", "replica_per_rank": True}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cl, wb = make_workload(args.workload, 0)
    kind, s, run = time_cpu(wb)
    for _ in range(args.warmup):
        run(s["batch"])
    ts = []
    for _ in range(args.steps):
        t = time.time()
        run(s["batch"])
        ts.append(time.time() - t)
    v = s["n_int"] / statistics.mean(ts) / 1e9
    out = {"metric": "tree-force Ginteractions/s at N=1M", "impl": "reference", "value": v,
           "unit": "Ginteractions/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * statistics.mean(ts), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": workload_config(args.workload, cl, wb), "sample": s["desc"],
           "cpu_baseline": {"value": v, "unit": "Ginteractions/s", "cores": os.cpu_count(), "kind": kind,
                            "sample": s["desc"]},
           "e2e": {"value": v, "unit": "Ginteractions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    from petar_gb300 import gpuforce, walks
    from petar_gb300.gpuforce import PGF_PRECISION_FP64, PGF_PRECISION_MIXED

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    cl, wb = make_workload(args.workload, rank)
    n_epep, n_epsp = wb.interactions()
    n_int = n_epep + n_epsp
    flops = FLOPS_EPEP * n_epep + FLOPS_EPSP * n_epsp
    rec = gpuforce.Records(wb)
    # A dedicated (non-default) stream: the library launches on it and the
    # CUDA events below are recorded on it.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    gpuforce.CalcForceWithLinearCutoffCUDAMultiWalk(local, wb.eps2, wb.rcut2, wb.G)
    gpuforce.set_stream(stream.cuda_stream)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2

    # ---- device-resident mixed-precision steps ----
    gpuforce.set_precision(PGF_PRECISION_MIXED)
    gpuforce.dispatch(rec, tag=0)
    gpuforce.retrieve(rec, tag=0)
    # The library's autotuner picks the kernel variant on this workload; each
    # variant's time is also recorded for the report.
    variant_ms = {}
    if args.variant >= 0:
        # fixed variant (profiling runs): no sweep, no autotuner
        gpuforce.set_kernel_variant(args.variant)
        best_variant = args.variant
    else:
        for v in range(gpuforce.NUM_KERNEL_VARIANTS):
            gpuforce.set_kernel_variant(v)
            gpuforce.recompute(0)
            gpuforce.wait(0)
            gpuforce.recompute(0)
            gpuforce.wait(0)
            variant_ms[v] = 1e3 * gpuforce.get_profile()["last_calc_main"]
        best_variant, _ = gpuforce.autotune(0, repeats=2)
    gpuforce.recompute(0)
    f_mixed = gpuforce.retrieve(rec, tag=0).copy()
    for _ in range(args.warmup):
        flush.zero_()
        gpuforce.recompute(0)
        gpuforce.wait(0)
    gpuforce.clear_profile()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    main_ms = []
    barrier()
    wall0 = time.time()
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    bus = getattr(props, "pci_bus_id", None)
    bus = f"{getattr(props, 'pci_domain_id', 0):08x}:{bus:02x}:{getattr(props, 'pci_device_id', 0):02x}.0" \
        if isinstance(bus, int) else bus
    with NvmlSampler(bus, torch.cuda.current_device()) as nv, ClockSampler(torch.cuda.current_device()) as clk:
        for e0, e1 in evs:
            flush.zero_()
            e0.record(stream)
            gpuforce.recompute(0)
            e1.record(stream)
            gpuforce.wait(0)
            main_ms.append(1e3 * gpuforce.get_profile()["last_calc_main"])
        barrier()
    wall = time.time() - wall0
    prof = gpuforce.get_profile()
    step_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    t_total = max_over_ranks(sum(step_ms) / 1e3, world)
    value = job_throughput(n_int, args.steps, t_total, world)
    clocks = nv.summary() or clk.summary()
    n_retest = prof["n_retest"] / max(1, prof["n_call"] or args.steps)

    # ---- plain FP64 kernel on the same lists ----
    fp64 = None
    f64 = None
    parity_violations: list[str] = []
    if not args.no_fp64:
        gpuforce.set_precision(PGF_PRECISION_FP64)
        gpuforce.recompute(0)
        f64 = gpuforce.retrieve(rec, tag=0).copy()
        ts = []
        for _ in range(max(1, min(2, args.steps))):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            gpuforce.recompute(0)
            e1.record(stream)
            gpuforce.wait(0)
            ts.append(e0.elapsed_time(e1))
        t64 = max_over_ranks(statistics.mean(ts) / 1e3, world)
        v64 = world * n_int / t64 / 1e9
        ea = np.linalg.norm(f_mixed["acc"] - f64["acc"], axis=1) / np.linalg.norm(f64["acc"], axis=1)
        ep = np.abs(f_mixed["pot"] - f64["pot"]) / np.abs(f64["pot"])
        fp64 = {"value": v64, "unit": "Ginteractions/s", "ms_per_step": 1e3 * t64, "speedup_mixed_vs_fp64": value / v64,
                "accuracy_mixed_vs_fp64": {
                    "force_rel_err_median": float(np.median(ea)), "force_rel_err_p999": float(np.quantile(ea, 0.999)),
                    "force_rel_err_max": float(ea.max()),
                    "pot_rel_err_median": float(np.median(ep)), "pot_rel_err_p999": float(np.quantile(ep, 0.999)),
                    "pot_rel_err_max": float(ep.max()),
                    "n_ngb_mismatches": int((f_mixed["n_ngb"] != f64["n_ngb"]).sum()),
                    "bounds": "median <= 1e-6, p99.9 <= 1e-5, max <= 1e-3, counts exact"}}
        parity_violations += accuracy_violations(fp64["accuracy_mixed_vs_fp64"])
        gpuforce.set_precision(PGF_PRECISION_MIXED)

    # ---- the reference's own CUDA kernels on the same lists ----
    ref_gpu = None
    if not args.no_fp64 and rank == 0:
        ref_gpu = reference_gpu_kernel(wb, n_int, f64)

    # ---- end to end through the C ABI with host records ----
    ni, ne, ns = wb.epi_rs.size, wb.id_epj.size, wb.id_spj.size
    # EPJ: EpjMix 32 B + FP64 mass and r_search 16 B; SPJ: SpjMix 64 B + SpjQ64 64 B;
    # EPI 32 B; ids 4 B; walk descriptor 96 B + queue entry 4 B.  Back: Accp
    # 32 B + count 4 B per i, and the 16-byte status words.
    h2d = (wb.epj_mass.size * 48 + wb.spj_mass.size * 128 + ni * 32 + (ne + ns) * 4 + wb.n_walk * 100)
    d2h = ni * (32 + 4) + 16
    # The library's dispatch autotuner: pipeline stages and split unit on
    # this workload's host records (kept for the e2e steps below).
    tuned_dispatch = gpuforce.autotune_dispatch(rec, tag=0, repeats=2)
    e2e_t = []
    for k in range(args.warmup + args.steps):
        barrier()
        if k == args.warmup:
            gpuforce.clear_profile()
        t = time.time()
        gpuforce.dispatch(rec, tag=0, send=True)
        gpuforce.retrieve(rec, tag=0)
        if k >= args.warmup:
            e2e_t.append(time.time() - t)
    e2e_total = max_over_ranks(sum(e2e_t), world)
    bd = gpuforce.get_profile()
    e2e = {"value": world * n_int * args.steps / e2e_total / 1e9, "unit": "Ginteractions/s",
           "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
           "ms_per_step": 1e3 * e2e_total / args.steps,
           "breakdown_ms_per_step": {k: 1e3 * bd[k] / args.steps for k in ("copy", "send", "calc", "recv")},
           "host_direct": gpuforce.host_direct_active(), "tuned_dispatch": tuned_dispatch}

    # ---- the other modes on the same lists ----
    modes = None
    if not args.no_modes:
        def time_recompute(tag: int, n: int = 3) -> float:
            ts = []
            for _ in range(n + 1):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                gpuforce.recompute(tag)
                e1.record(stream)
                gpuforce.wait(tag)
                ts.append(e0.elapsed_time(e1))
            return statistics.mean(ts[1:])
        modes = {}
        # neighbour search (SearchNeighborEpEp): EP-EP lists only
        gpuforce.set_mode(gpuforce.PGF_MODE_NEIGHBOR_SEARCH)
        try:
            gpuforce.dispatch(rec, tag=1, send=False)
            gpuforce.retrieve(rec, tag=1)
            t = time_recompute(1)
        finally:
            gpuforce.set_mode(gpuforce.PGF_MODE_FORCE)
        modes["neighbor_search"] = {"ms_per_step": t, "value": n_epep / t / 1e6, "unit": "Gpairs/s",
                                    "pairs": n_epep}
        # soft force with the changeover correction of neighbours fused in
        wb_co, co = walks.make_changeover(wb, cl.r_in, cl.r_out, seed=1)
        rec_co = gpuforce.Records(wb_co, co)
        gpuforce.set_changeover_layout(rec_co)
        gpuforce.set_mode(gpuforce.PGF_MODE_FORCE_CHANGEOVER)
        try:
            gpuforce.dispatch(rec_co, tag=2)
            gpuforce.retrieve(rec_co, tag=2)
            t = time_recompute(2)
        finally:
            gpuforce.set_mode(gpuforce.PGF_MODE_FORCE)
            gpuforce.set_changeover_layout(None)
        co_entry = {"ms_per_step": t, "value": n_int / t / 1e6, "unit": "Ginteractions/s",
                    "overhead_vs_force_mode": t / statistics.mean(step_ms),
                    "members_fraction": 0.1, "artificial_fraction": 0.05,
                    "parity": "tests/test_gpu_parity.py::test_changeover_mode_*"}
        modes["force_changeover"] = co_entry
        # KDKDK_4TH gradient-correction pass, with the force pass's accelerations
        acc = f_mixed["acc"]
        rec_gr = gpuforce.Records(wb, acc=(acc, acc))
        gpuforce.set_gradient_layout(rec_gr)
        gpuforce.set_mode(gpuforce.PGF_MODE_GRADIENT)
        try:
            t_mode = {}
            for acc_mode in (0, 1):  # plain FP32 far pairs, then the default compensated ones
                gpuforce.set_gradient_accuracy(acc_mode)
                gpuforce.dispatch(rec_gr, tag=3)
                gpuforce.retrieve(rec_gr, tag=3)
                t_mode[acc_mode] = time_recompute(3)
            t = t_mode[1]
        finally:
            gpuforce.set_gradient_accuracy(1)
            gpuforce.set_mode(gpuforce.PGF_MODE_FORCE)
            gpuforce.set_gradient_layout(None)
        modes["gradient_kdkdk"] = {"ms_per_step": t, "value": n_int / t / 1e6, "unit": "Ginteractions/s",
                                   "accuracy_mode": "compensated (default)",
                                   "fp32_far_pairs_ms_per_step": t_mode[0],
                                   "parity": "tests/test_gpu_parity.py::test_gradient_mode_*"}

    # ---- the other named configurations: Plummer 65k and the 64-cluster ensemble ----
    # (rank 0 only: the other ranks' lines are not printed)
    configs = None
    if not args.no_configs and rank == 0:
        configs = {"fdps_batches_200": run_fdps_batches(wb, rec, n_int)}
        configs.update(run_configs(stream, flush))
        gpuforce.set_precision(PGF_PRECISION_MIXED)

    # ---- device-resident tree step: King W0=7, 4M, 100 KDK steps in one CUDA graph ----
    kdk = None
    if not args.no_kdk and rank == 0:
        kdk = run_kdk_graph()

    if rank != 0:
        torch.distributed.barrier()
        return

    # ---- roofline of the main kernel ----
    peaks = fp32_peak_tflops()
    peak = max(v for v in peaks.values() if v) if any(peaks.values()) else None
    main_s = statistics.mean(main_ms) / 1e3
    achieved = flops / main_s / 1e12
    kernel_name = "mixed_kernel" if best_variant == 0 else f"ws_kernel (variant {best_variant})"
    roof = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak if peak else None, "traffic": traffic_from_profiles(),
            "peak_source": "FP32 FMA loops measured in this run, the faster of scalar and packed FP32x2 "
                           "(MEASURED_PEAKS.json has no FP32 figure)", "peaks_measured": peaks,
            "flops_per_launch": flops, "kernel": kernel_name, "launch_ms": 1e3 * main_s,
            "flop_model": "19 per EP-EP, 54 per EP-SP interaction"}

    cpu = None
    if world == 1 and not args.no_cpu:
        kind, s, run = time_cpu(wb)
        t = time.time()
        run(s["batch"])
        dt = time.time() - t
        cpu = {"value": s["n_int"] / dt / 1e9, "unit": "Ginteractions/s", "cores": os.cpu_count(),
               "kind": kind, "sample": s["desc"], "seconds": dt}

    out = {
        "metric": "tree-force Ginteractions/s at N=1M", "value": value, "unit": "Ginteractions/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic",
        "config": workload_config(args.workload, cl, wb),
        "gpu_launches": 2 * args.steps,
        "kernel_variant": best_variant, "variant_main_ms": variant_ms,
        "fp64_plain": fp64, "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clocks,
        "retest_records_per_step": n_retest, "wall_s_timed_region": wall, "modes": modes,
        "kdk_graph": kdk, "configs": configs, "reference_gpu_kernel": ref_gpu,
        "cpu_reference_x86": cpu_reference_x86(),
    }
    if parity_violations:
        out["parity_violations"] = parity_violations
    print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.barrier()
    if parity_violations:
        # A throughput whose results miss the parity bar is not a result.
        log("parity violated: " + "; ".join(parity_violations))
        sys.exit(3)


def reference_gpu_kernel(wb, n_int: int, f64) -> dict:
    """The reference's force_kernel_ep_ep + force_kernel_ep_sp (compiled from
    its sources into a cubin, launched as its functor launches them) on the
    same lists: kernel time and accuracy against the plain FP64 kernel."""
    import oracle
    try:
        r = oracle.ref_gpu(wb, repeats=3)
    except oracle.ReferenceKernelUnavailable as e:
        return {"unavailable": str(e)}
    out = {"ms_per_step": r["ms"], "value": n_int / r["ms"] / 1e6, "unit": "Ginteractions/s",
           "kernels": "force_kernel_ep_ep + force_kernel_ep_sp (src/force_gpu_cuda.cu), one launch each, all walks"}
    if f64 is not None:
        ea = np.linalg.norm(r["acc"] - f64["acc"], axis=1) / np.linalg.norm(f64["acc"], axis=1)
        ep = np.abs(r["pot"] - f64["pot"]) / np.abs(f64["pot"])
        out["accuracy_vs_fp64"] = {
            "force_rel_err_median": float(np.median(ea)), "force_rel_err_p999": float(np.quantile(ea, 0.999)),
            "force_rel_err_max": float(ea.max()), "pot_rel_err_median": float(np.median(ep)),
            "pot_rel_err_p999": float(np.quantile(ep, 0.999)), "pot_rel_err_max": float(ep.max()),
            "n_ngb_mismatches": int((r["nnb"] != f64["n_ngb"]).sum())}
    return out


def cpu_reference_x86() -> dict | None:
    """The reference's AVX-512 CPU kernels (PhantomGrapeQuad FP32 and 64-bit)
    and FP64 NoSimd functors on the same seeded sample of this workload,
    measured on an x86 host by oracle/ref/time_cpu_reference.py (the GPU hosts
    are aarch64): a side record read from its committed summary."""
    p = ROOT / "profiles" / "cpu_reference_x86_plummer1m_bin50.md"
    if not p.exists():
        return None
    m = re.search(r"^record: (\{.*\})$", p.read_text(), flags=re.M)
    return json.loads(m.group(1)) if m else None


def run_fdps_batches(wb, rec, n_int: int, batch: int = 200, reps: int = 3) -> dict:
    """The bench workload through the functors as PeTar calls them unchanged:
    FDPS hands over n_walk_limit = 200 walks per call (src/petar.hpp:888)
    with one tag, so each batch is dispatched and retrieved before the next
    (send once, then 55 dispatch/retrieve pairs), with and without walk
    splitting.  Host records, copies and unpacking included."""
    from petar_gb300 import gpuforce
    gpuforce.set_precision(gpuforce.PGF_PRECISION_MIXED)
    f = gpuforce.CalcForceWithLinearCutoffCUDAMultiWalk(0, rec.eps2, rec.rcut2, rec.G)
    nw = rec.n_walk

    def one_eval():
        f(0, 0, None, None, None, None, None, None, rec.epj, rec.epj.size, rec.spj, rec.spj.size, True)
        for w0 in range(0, nw, batch):
            w1 = min(nw, w0 + batch)
            f(0, w1 - w0, rec.p_epi[w0:w1], rec.n_epi[w0:w1], rec.p_id_epj[w0:w1], rec.n_epj[w0:w1],
              rec.p_id_spj[w0:w1], rec.n_spj[w0:w1], None, 0, None, 0, False, epi_dtype=rec.epi.dtype)
            gpuforce.RetrieveForceCUDA(0, w1 - w0, rec.n_epi[w0:w1], rec.p_force[w0:w1],
                                       force_dtype=rec.force.dtype)

    out = {"walks_per_call": batch, "calls_per_evaluation": (nw + batch - 1) // batch, "unit": "Ginteractions/s",
           "caller": "the Python functors (ctypes)"}
    # The dispatch autotuner on one 200-walk call from the middle of the
    # evaluation (the split unit matters for calls this small).
    mid = nw // 2 // batch * batch
    sub = walks_subset_records(rec, mid, min(nw, mid + batch))
    out["tuned_dispatch"] = gpuforce.autotune_dispatch(sub, tag=0, repeats=3)
    try:
        for split in (True, False):
            gpuforce.set_walk_split(split)
            one_eval()
            ts = []
            for _ in range(reps):
                t = time.time()
                one_eval()
                ts.append(time.time() - t)
            key = "split" if split else "no_split"
            out[key] = {"ms_per_evaluation": 1e3 * min(ts), "value": n_int / min(ts) / 1e9}
    finally:
        gpuforce.set_walk_split(True)
    out["cpp_functors"] = fdps_batches_cpp(wb, n_int, batch)
    return out


def fdps_batches_cpp(wb, n_int: int, batch: int = 200, reps: int = 3) -> dict:
    """The same call pattern from C++ (bench_support/fdps_batches.cpp): the
    header functors with PeTar-layout records, as PeTar itself calls them,
    with no Python between the calls; checked against the single-dispatch
    result of the same lists."""
    import ctypes
    from bench_support import build_fdps_driver
    from petar_gb300 import gpuforce
    lib = ctypes.CDLL(str(build_fdps_driver()))
    vp = ctypes.c_void_p
    lib.fdps_batches_run.argtypes = ([ctypes.c_int64, vp, vp, vp, vp, vp, ctypes.c_int64, vp, vp, vp,
                                      ctypes.c_int64, vp, vp, vp, vp, vp] + [ctypes.c_double] * 3
                                     + [ctypes.c_int, ctypes.c_int, vp, vp, vp, vp])
    lib.fdps_batches_run.restype = ctypes.c_int
    c = lambda a, t: np.ascontiguousarray(a, dtype=t)
    arrs = [c(wb.n_epi, np.int32), c(wb.n_epj, np.int32), c(wb.n_spj, np.int32), c(wb.epi_pos, np.float64),
            c(wb.epi_rs, np.float64)]
    je = [c(wb.epj_mass, np.float64), c(wb.epj_pos, np.float64), c(wb.epj_rs, np.float64)]
    js = [c(wb.spj_mass, np.float64), c(wb.spj_pos, np.float64), c(wb.spj_quad, np.float64)]
    ids = [c(wb.id_epj, np.int32), c(wb.id_spj, np.int32)]
    ni = wb.epi_rs.size
    acc, pot, nnb = np.zeros((ni, 3)), np.zeros(ni), np.zeros(ni, np.int64)
    ms = ctypes.c_double()
    rc = lib.fdps_batches_run(wb.n_walk, *[a.ctypes.data for a in arrs], wb.epj_mass.size,
                              *[a.ctypes.data for a in je], wb.spj_mass.size, *[a.ctypes.data for a in js],
                              *[a.ctypes.data for a in ids], wb.eps2, wb.rcut2, wb.G, batch, reps,
                              ctypes.byref(ms), acc.ctypes.data, pot.ctypes.data, nnb.ctypes.data)
    if rc != 0:
        return {"error": f"driver returned {rc}"}
    ref = gpuforce.compute(wb, gpuforce.PGF_PRECISION_MIXED)
    ea = np.linalg.norm(acc - ref["acc"], axis=1) / np.linalg.norm(ref["acc"], axis=1)
    return {"ms_per_evaluation": ms.value, "value": n_int / ms.value / 1e6, "unit": "Ginteractions/s",
            "caller": "C++ (bench_support/fdps_batches.cpp, include/petar_gpuforce.hpp)",
            "vs_single_dispatch": {"force_rel_err_p999": float(np.quantile(ea, 0.999)),
                                   "n_ngb_mismatches": int((nnb != ref["nnb"]).sum())}}


def walks_subset_records(rec, w0: int, w1: int):
    """A Records view of walks [w0, w1): the same j arrays and pointer tables."""
    import copy
    sub = copy.copy(rec)
    sub.n_walk = w1 - w0
    for k in ("n_epi", "n_epj", "n_spj", "p_epi", "p_force", "p_id_epj", "p_id_spj"):
        setattr(sub, k, np.ascontiguousarray(getattr(rec, k)[w0:w1]))
    sub.walk_rcut2 = None if rec.walk_rcut2 is None else rec.walk_rcut2[w0:w1]
    return sub


def _time_tag(tag: int, stream, flush, reps: int = 3) -> float:
    """Mean event time (ms) of re-running a tag's kernels on resident data,
    the L2 flushed before each run; the first run is a warm-up."""
    import torch
    from petar_gb300 import gpuforce
    ts = []
    for _ in range(reps + 1):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        gpuforce.recompute(tag)
        e1.record(stream)
        gpuforce.wait(tag)
        ts.append(e0.elapsed_time(e1))
    return statistics.mean(ts[1:])


def run_configs(stream, flush) -> dict:
    """Plummer N = 65,536 (theta 0.3, r_out 0.008): mixed against the plain
    FP64 kernel on the same lists.  Ensemble: 64 Plummer clusters, N
    log-uniform in [1024, 65536], 30% binaries, r_out = 0.05 N^(-1/3), all
    walks in one mixed-precision launch against 64 sequential launches of the
    plain FP64 kernel (and of the mixed one), one per cluster."""
    from petar_gb300 import gpuforce, ics, walks
    from petar_gb300.gpuforce import PGF_PRECISION_FP64, PGF_PRECISION_MIXED
    out = {}
    tag = 4
    cl = ics.make_plummer_cluster(2, 65536, 0.008)
    wb = walks.build_walks(cl)
    rec = gpuforce.Records(wb)
    n = sum(wb.interactions())
    t = {}
    for prec in (PGF_PRECISION_MIXED, PGF_PRECISION_FP64):
        gpuforce.set_precision(prec)
        gpuforce.dispatch(rec, tag=tag)
        gpuforce.retrieve(rec, tag=tag)
        t[prec] = _time_tag(tag, stream, flush)
    out["plummer65k"] = {"n": int(cl.n), "n_walk": int(wb.n_walk), "interactions": int(n),
                         "mixed_ms": t[PGF_PRECISION_MIXED], "fp64_ms": t[PGF_PRECISION_FP64],
                         "mixed_value": n / t[PGF_PRECISION_MIXED] / 1e6, "fp64_value": n / t[PGF_PRECISION_FP64] / 1e6,
                         "unit": "Ginteractions/s", "speedup_mixed_vs_fp64": t[PGF_PRECISION_FP64] / t[PGF_PRECISION_MIXED],
                         "parity": "tests/test_gpu_configs.py::test_plummer65k_against_oracle_and_direct_sum"}
    rng = np.random.default_rng(5)
    ns = np.round(np.exp(rng.uniform(np.log(1024), np.log(65536), 64))).astype(int)
    bs = []
    for k, nk in enumerate(ns):
        c = ics.make_plummer_cluster(500 + k, int(nk), 0.05 * nk ** (-1 / 3), binary_fraction=0.3)
        b = walks.build_walks(c)
        b.walk_rcut2 = np.full(b.n_walk, c.r_out ** 2)
        bs.append(b)
    seq = {PGF_PRECISION_MIXED: 0.0, PGF_PRECISION_FP64: 0.0}
    for b in bs:
        r = gpuforce.Records(b)
        for prec in seq:
            gpuforce.set_precision(prec)
            gpuforce.dispatch(r, tag=tag)
            gpuforce.retrieve(r, tag=tag)
            seq[prec] += _time_tag(tag, stream, flush, reps=1)
    wbe = walks.concat_batches(bs)
    r = gpuforce.Records(wbe)
    gpuforce.set_precision(PGF_PRECISION_MIXED)
    gpuforce.dispatch(r, tag=tag)
    gpuforce.retrieve(r, tag=tag)
    t1 = _time_tag(tag, stream, flush)
    n = sum(wbe.interactions())
    out["ensemble64"] = {"n_clusters": 64, "n": int(sum(ns)), "n_walk": int(wbe.n_walk), "interactions": int(n),
                         "mixed_one_launch_ms": t1, "fp64_64_launches_ms": seq[PGF_PRECISION_FP64],
                         "mixed_64_launches_ms": seq[PGF_PRECISION_MIXED], "mixed_value": n / t1 / 1e6,
                         "unit": "Ginteractions/s",
                         "speedup_vs_64_fp64_launches": seq[PGF_PRECISION_FP64] / t1,
                         "speedup_vs_64_mixed_launches": seq[PGF_PRECISION_MIXED] / t1,
                         "parity": "tests/test_gpu_configs.py::test_ensemble64_one_launch"}
    return out


def run_kdk_graph(n: int = 4194304, steps: int = 100, dt: float = 1.0 / 1024) -> dict:
    """The King W0 = 7 configuration as a device-resident run: tree, lists,
    force, kicks and drifts of `steps` leapfrog steps in one CUDA graph.
    Throughput counts the interactions of every step's lists over the graph's
    device time (tree building included)."""
    from petar_gb300 import ics, nbody
    clk = ics.make_king_cluster(7, n, 0.0015, W0=7.0, theta=0.4)
    rng = np.random.default_rng(11)
    sample = np.sort(rng.choice(n, 4096, replace=False))
    with nbody.DeviceNBody(clk) as h:
        # n_group_limit autotuner (tree + lists + force per evaluation), then
        # the kernel variant for the chosen lists.
        groups = h.autotune_groups((256, 512, 1024, 2048), repeats=2)
        variant, _ = h.autotune(2)
        # Accuracy run: every step records a random 4096-particle sample, mixed
        # precision against an FP64 evaluation over the same lists.
        h.set_sample(sample, steps + 1)
        h.force()
        st0 = h.stats()
        e0 = sum(h.energy())
        h.run(steps, dt, graph=True)
        e1 = sum(h.energy())
        recs = h.samples()
        # Timed runs without the sample: capture, then the replay is timed.
        h.set_sample(np.zeros(0, np.int64), 0)
        h.run(steps, dt, graph=True)
        st1 = h.stats()
        ms = h.run(steps, dt, graph=True)
        st2 = h.stats()
    inter = (st2["total_epep"] - st1["total_epep"]) + (st2["total_epsp"] - st1["total_epsp"])
    per_step = []
    for r in recs:
        ea = np.linalg.norm(r["acc"] - r["acc64"], axis=1) / np.linalg.norm(r["acc64"], axis=1)
        ep = np.abs(r["pot"] - r["pot64"]) / np.abs(r["pot64"])
        per_step.append((float(np.median(ea)), float(np.quantile(ea, 0.999)), float(np.median(ep)),
                         float(np.quantile(ep, 0.999)), int((r["n_ngb"] != r["n_ngb64"]).sum())))
    ps = np.array(per_step)
    return {"config": {"model": "King W0=7", "n": n, "theta": 0.4, "r_out": 0.0015, "dt": dt,
                       "n_leaf_limit": clk.n_leaf_limit, "n_group_limit": groups["best_n_group_limit"]},
            "group_limit_autotune": groups,
            "steps_per_graph": steps, "ms_per_step": ms / steps, "value": inter / (ms * 1e-3) / 1e9,
            "unit": "Ginteractions/s over whole steps (tree, lists, force, kicks, drifts)",
            "tree_ms": st0["last_tree_ms"], "force_ms": st0["last_force_ms"],
            "interactions_per_step": inter / steps, "n_groups": st0["n_groups"], "n_cells": st0["n_cells"],
            "energy_rel_change": (e1 - e0) / abs(e0), "kernel_variant": variant,
            "per_step_error_vs_fp64": {
                "sample": "4096 random particles, every one of the %d force evaluations" % len(per_step),
                "reference": "FP64 evaluation of the same lists on the device (pinned to the oracle in tests)",
                "force_rel_err_median_max_over_steps": float(ps[:, 0].max()),
                "force_rel_err_p999_max_over_steps": float(ps[:, 1].max()),
                "pot_rel_err_median_max_over_steps": float(ps[:, 2].max()),
                "pot_rel_err_p999_max_over_steps": float(ps[:, 3].max()),
                "n_ngb_mismatches_total": int(ps[:, 4].sum())},
            "parity": "tests/test_gpu_nbody.py"}


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="plummer1m_bin50")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-modes", action="store_true", help="skip the search and changeover mode timings")
    ap.add_argument("--no-kdk", action="store_true", help="skip the device-resident King 4M KDK run")
    ap.add_argument("--no-configs", action="store_true", help="skip the Plummer 65k and ensemble timings")
    ap.add_argument("--variant", type=int, default=-1,
                    help="use this kernel variant instead of the autotuner's choice")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        log("note: fewer than 3 warm-up steps")
    if args.impl == "reference":
        run_reference(args)
    else:
        from petar_gb300.build import build_all
        build_all()
        run_ours(args)


if __name__ == "__main__":
    main()
