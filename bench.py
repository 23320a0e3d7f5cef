"""Benchmark: 2.5D complex-resistivity forward + Jacobian units per second.

One unit (a "step") is the complete forward -- every wavenumber x current
electrode assembled, factorised and solved, back-transformed, voltages -- plus
the full Jacobian (src/bsens.f90), for one conductivity model.  The workload
is the 200x60-quad, 96-electrode, 4000-quadrupole configuration (synthetic,
seeded; titatest_gb300.synth.config2).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
  python bench.py --case --config C [--batch B] [--sens] ...   (one forward, for ncu)

value : mixed mode (complex64 factor + FP64 refinement), inputs resident on
        the device, timed with CUDA events on the library's stream;
e2e   : the same unit through the host C ABI (crgpu_forward + crgpu_sens with
        pinned host buffers: sigma in, voltages and the Jacobian out), with
        d2h_link_gbs, the rate of a plain pinned copy of the Jacobian's bytes
        in the same run (the host link is shared and its rate varies);
plain : the complex128 mode on the same inputs (the reference arithmetic),
        with the mixed/plain speed-up and the error of mixed against plain.
--impl reference times the oracle (the plain-C restatement of the reference
routines, OpenMP over all host cores) on whole units of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "2.5D CR forward+Jacobian/s, mixed vs FP64 plain at 1e-6 rel err; % roofline"


def _dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def tensor_peak_tflops():
    """Dense tensor peak for a kernel timed inside a long step: the sustained
    bf16 figure of MEASURED_PEAKS.json (measured on this machine), else
    the fallback measurement of 1.7 PFLOP/s."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["bf16_tflops_sustained"]), "MEASURED_PEAKS.json bf16_tflops_sustained (of measured)"
    except (OSError, KeyError, ValueError):
        return 1700.0, "fallback 1.7 PFLOP/s sustained bf16 (of fallback)"


def fp64_dgemm_tflops(stream) -> float:
    """The FP64 rate of this GPU as cuBLAS DGEMM reaches it (4096^3, best of
    3, CUDA events): the denominator of the complex128 factor's roofline."""
    import torch
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = float("inf")
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        torch.matmul(a, b)
        e1.record(stream)
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * 4096 ** 3 / (best * 1e-3) / 1e12


def hbm_peak_gbs():
    """The copy bandwidth of MEASURED_PEAKS.json (measured on this
    pool), else the fallback 6.8 TB/s."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (of measured)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s (of fallback)"


def fp32_sgemm_tflops(stream) -> float:
    """The FP32 FMA-pipe rate of this GPU as cuBLAS SGEMM reaches it (TF32
    off, 8192^3, best of 3, CUDA events): the denominator of the SIMT
    complex64 factor kernels' roofline."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        a = torch.randn(8192, 8192, dtype=torch.float32, device="cuda")
        b = torch.randn(8192, 8192, dtype=torch.float32, device="cuda")
        torch.matmul(a, b)
        best = float("inf")
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            torch.matmul(a, b)
            e1.record(stream)
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    return 2.0 * 8192 ** 3 / (best * 1e-3) / 1e12


def factored_band(m, g) -> int:
    """Band width of the matrix a context factors: the grid's, or that of its
    geometric node order (crgpu_node_order)."""
    order = np.asarray(m.node_order(), dtype=np.int64) - 1  # grid node at each position
    pos = np.empty(g.sanz, np.int64)
    pos[order] = np.arange(g.sanz)
    area = np.asarray(g.nrel[: g.nelanz[0]], dtype=np.int64) - 1
    p = pos[area]
    return int((p.max(axis=1) - p.min(axis=1)).max())


FACTOR_KERNELS = {"tensor cores": ("k_factor_tc", "tensor"), "SIMT warp per system": ("k_factor_warp", "fp32"),
                  "SIMT register tiles": ("k_factor_mixed", "fp32"),
                  "SIMT shared-memory tiles": ("k_factor_mixed_smem", "fp32")}


FACTOR_NOTES = {
    "k_factor_warp": "latency-bound band factor: a serial chain per column (pivot, reciprocal, rank-1 update of "
                     "the 64-slot window held in one warp's registers), one system per warp, 12 warps an SM",
    "k_factor_warp2": "latency-bound band factor, two columns a step (2x2 pivot block, two rank-1 updates of the "
                      "64-slot window held in one warp's registers), one system per warp, 8 warps an SM; the "
                      "systems beyond 8 an SM are factored on the tensor cores beside the solves",
    "k_factor_tc": "latency-bound band factor: each 4-column step is a serial panel plus 4 tf32 MMAs (3 hi/lo "
                   "products + row injection) on a 128x128 complex window"}


def read_profile_traffic(name: str):
    """DRAM bytes per launch recorded from an ncu capture (profiles/<name>)."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_launch_full_workload:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (plain-C restatement, OpenMP) on whole units
# ---------------------------------------------------------------------------
def oracle_unit(P, sigma, kwn, kwnwi, threads):
    """One whole unit on the oracle's timing build: the forward of every
    (k, l) system with OpenMP over the wavenumbers (src/fem.f90:257-277,
    327-397: at most kwnanz threads), rtrafo, bvolt, and bsens over every
    measurement with OpenMP over the measurements (src/bsens.f90:94-100).
    Returns (volt, sens (nanz, elanz) view, forward seconds, sens seconds)."""
    t0 = time.perf_counter()
    kp = P.forward(sigma, kwn, kwnwi, nthreads=threads)
    hp = P.rtrafo(kp, kwnwi)
    volt, _ = P.bvolt(hp, 0, None)
    t1 = time.perf_counter()
    sens = P.bsens(kp, kwn, kwnwi, sigma, volt, mode=0, nthreads=threads, contiguous=False)
    t2 = time.perf_counter()
    return volt, sens, t1 - t0, t2 - t1


def cpu_baseline(s, kwn, kwnwi, threads=None, units=1):
    """The oracle timed on `units` whole units of the workload (no sampling,
    no scaling): forward on its own potentials, then the full Jacobian."""
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    P = O.Problem(s.grid, s.survey, timing=True)
    fw, sj = [], []
    for _ in range(units):
        _, _, tf, ts = oracle_unit(P, s.sigma, kwn, kwnwi, threads)
        fw.append(tf)
        sj.append(ts)
    unit_s = (sum(fw) + sum(sj)) / units
    nsys = len(kwn) * s.survey.eanz
    return {"value": 1.0 / unit_s, "unit": "units/s", "cores": threads, "kind": "port",
            "sample": (f"{units} whole unit(s): all {nsys} (k,l) systems (OpenMP over the {len(kwn)} wavenumbers, "
                       f"as src/fem.f90) and all {s.survey.nanz} Jacobian rows (OpenMP over measurements, as "
                       f"src/bsens.f90); oracle built with the reference's -O3 -ffast-math flags"),
            "seconds_per_unit": unit_s, "forward_s": statistics.mean(fw), "sens_s": statistics.mean(sj)}


def workload_string(cfg: int, s, K: int) -> str:
    g, sv = s.grid, s.survey
    kind = "triangles" if getattr(s, "triangles", False) else "quads"
    nsys = K * sv.eanz
    return (f"config{cfg}: {g.elanz} {kind}, {g.sanz} nodes, mb={g.mb}, {sv.eanz} electrodes, "
            f"{sv.nanz} quadrupoles, {K} wavenumbers ({nsys} band systems)")


def _product_library_mapped() -> bool:
    """True when libcrtomo_gb300.so is mapped into this process."""
    try:
        with open("/proc/self/maps") as f:
            return any("libcrtomo_gb300" in line for line in f)
    except OSError:
        return False


def workload_config(cfg: int, s, K: int) -> dict:
    """The `config` object of both arms (identical for the same workload)."""
    g, sv = s.grid, s.survey
    nsys = K * sv.eanz
    return {"workload": workload_string(cfg, s, K),
            "l2": "inputs larger than L2: the band factors of all %d systems are %.1f GB in complex64"
                  % (nsys, nsys * g.sanz * (g.mb + 1) * 8 / 1e9)}


def run_reference(args):
    """The reference arm: the oracle port of the reference routines (the
    Fortran reference cannot be built without a Fortran compiler) on whole
    units of the same workload, on the host cores.  The inputs come from the
    same seeded generator as the GPU arm, renumbered by the oracle's own
    CutMcK; no part of the GB300 library is loaded (checked below)."""
    rank, world, _ = _dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    from titatest_gb300 import synth  # numpy input generator; cutmck from the oracle
    threads = os.cpu_count() or 1
    s = synth.make(args.config, cutmck=O.cutmck)
    P = O.Problem(s.grid, s.survey, timing=True)
    kwn, kwnwi = P.rwaven()
    for _ in range(args.warmup):
        oracle_unit(P, s.sigma, kwn, kwnwi, threads)
    fw, sj = [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, _, tf, ts = oracle_unit(P, s.sigma, kwn, kwnwi, threads)
        fw.append(tf)
        sj.append(ts)
    wall = time.perf_counter() - t0
    v = args.steps / wall
    mapped = _product_library_mapped()
    if mapped:
        raise RuntimeError("the GB300 library was loaded into the reference arm")
    nsys = len(kwn) * s.survey.eanz
    cb = {"value": v, "unit": "units/s", "cores": threads, "kind": "port",
          "sample": (f"{args.steps} whole units: all {nsys} (k,l) systems (OpenMP over the {len(kwn)} wavenumbers, "
                     f"as src/fem.f90) and all {s.survey.nanz} Jacobian rows (OpenMP over measurements, as "
                     f"src/bsens.f90) per unit"),
          "seconds_per_unit": wall / args.steps, "forward_s": statistics.mean(fw), "sens_s": statistics.mean(sj)}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "units/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (seeded model and survey with the configuration's shapes)",
            "config": workload_config(args.config, s, len(kwn)),
            "parallelism": f"OpenMP {threads} threads (host cores)",
            "cpu_baseline": cb, "product_library_mapped": mapped,
            "build": "oracle/crt_oracle.c with -O3 -ftree-vectorize -ffast-math -finline-functions -fopenmp",
            "e2e": {"value": v, "unit": "units/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gpu(args):
    import torch

    rank, world, local = _dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from titatest_gb300 import MIXED, PLAIN, CRMod, synth
    from titatest_gb300 import _lib

    s = synth.make(args.config)
    g, sv = s.grid, s.survey
    nanz, manz = sv.nanz, g.elanz
    stream = torch.cuda.current_stream()
    sig_dev = torch.from_numpy(s.sigma.view(np.float64).copy()).cuda()
    volt_dev = torch.zeros(2 * nanz, dtype=torch.float64, device="cuda")
    sens_dev = torch.zeros(2 * nanz * manz, dtype=torch.float64, device="cuda")

    mixed = CRMod(g, sv, precision=MIXED, band_order=args.band_order)
    mixed.set_stream(stream.cuda_stream)
    mixed.set_refinement(args.refine_maxit, args.refine_tol)
    tune = mixed.autotune(s.sigma) if not args.no_autotune else mixed.tune()
    K = mixed.kwnanz

    def unit(m):
        m.forward_device(sig_dev.data_ptr(), volt_dev.data_ptr())
        m.sens_device(0, sens_dev.data_ptr())

    def unit_graph(m):  # the same unit replayed as one CUDA graph (recorded on the first call)
        m.forward_sens_graph(sig_dev.data_ptr(), volt_dev.data_ptr(), 0, sens_dev.data_ptr())

    timed_unit = unit if args.no_graph else unit_graph
    for _ in range(args.warmup):
        timed_unit(mixed)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fac_ms, sens_ms, launches, iters = [], [], 0, []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            timed_unit(mixed)
            st = mixed.stats()
            iters.append(st["refine_iterations"])
            launches += st["kernel_launches"]
        ev1.record(stream)
        torch.cuda.synchronize()
    elapsed_ms = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([elapsed_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    ms_per_step = elapsed_ms / args.steps
    value = world * 1e3 / ms_per_step
    volt_mixed = volt_dev.cpu().numpy().view(np.complex128).copy()
    sens_mixed = sens_dev.cpu().numpy().view(np.complex128).copy()
    # per-phase figures (a replayed graph measures none): ordinary units
    for _ in range(2):
        unit(mixed)
        st = mixed.stats()
        fac_ms.append(st["ms_factor"])
        sens_ms.append(st["ms_sens"])

    # ---- e2e through the host C ABI with pinned buffers
    L = _lib.lib()
    h_sig = torch.from_numpy(s.sigma.view(np.float64).copy()).pin_memory()
    h_volt = torch.zeros(2 * nanz, dtype=torch.float64).pin_memory()
    h_sens = torch.zeros(2 * nanz * manz, dtype=torch.float64).pin_memory()
    import ctypes as C

    def unit_host():
        rc = L.crgpu_forward(mixed._h, C.c_void_p(h_sig.data_ptr()), None, None, 0, None,
                             C.c_void_p(h_volt.data_ptr()), None)
        rc = rc or L.crgpu_sens(mixed._h, 0, C.c_void_p(h_sens.data_ptr()))
        if rc:
            raise RuntimeError(f"C ABI error {rc}: {L.crgpu_last_error(mixed._h).decode()}")

    unit_host()
    torch.cuda.synchronize()
    e_steps = max(1, min(args.steps, 3))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e_steps):
        unit_host()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / e_steps
    h2d = 16 * manz
    d2h = 16 * nanz + 16 * nanz * manz
    # the host link's own rate for the Jacobian's bytes (a plain pinned copy),
    # so that the e2e figure can be read against what the link gave this run
    h_sens.copy_(sens_dev, non_blocking=True)
    e0.record(stream)
    for _ in range(e_steps):
        h_sens.copy_(sens_dev, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    link_gbs = 16 * nanz * manz * e_steps / (e0.elapsed_time(e1) * 1e6)

    # ---- plain complex128 on the same inputs
    mixed_stats = mixed.stats()
    plain = CRMod(g, sv, precision=PLAIN, band_order=args.band_order)
    plain.set_stream(stream.cuda_stream)
    unit(plain)  # warm-up
    torch.cuda.synchronize()
    p_steps = max(1, args.plain_steps)
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for _ in range(p_steps):
        unit(plain)
    p1.record(stream)
    torch.cuda.synchronize()
    plain_ms = p0.elapsed_time(p1) / p_steps
    plain_stats = plain.stats()
    volt_plain = volt_dev.cpu().numpy().view(np.complex128).copy()
    sens_plain = sens_dev.cpu().numpy().view(np.complex128).copy()
    err_v = float(np.abs(volt_mixed - volt_plain).max() / np.abs(volt_plain).max())
    err_j = float(np.abs(sens_mixed - sens_plain).max() / np.abs(sens_plain).max())
    plain.close()

    # ---- roofline of the dominant kernel (the complex64 band factorisation of
    #      the band the context factors); algorithmic work = complex L L^T of
    #      every system, 4 n mb^2 flops
    n, mb = g.sanz, g.mb
    mb_mixed = factored_band(mixed, g)
    nsys = K * sv.eanz
    flops_factor = nsys * 4.0 * n * mb * mb  # the grid's band: the complex128 arm factors it
    kname, bound = FACTOR_KERNELS.get(tune["factor"], ("k_factor_tc", "tensor"))
    nsys_main = nsys
    if kname == "k_factor_warp":
        # the library's split: up to 8 systems an SM in the timed factor launch,
        # the excess (at most one an SM) on the tensor cores beside the solves
        nsm = torch.cuda.get_device_properties(0).multi_processor_count
        if 0 < nsys - 8 * nsm <= nsm:
            nsys_main = 8 * nsm
        if mb_mixed <= 62:
            kname = "k_factor_warp2"
    flops_mixed = nsys_main * 4.0 * n * mb_mixed * mb_mixed
    fp64_peak = fp64_dgemm_tflops(stream)
    fac_avg_ms = statistics.mean(fac_ms)
    achieved = flops_mixed / (fac_avg_ms * 1e-3) / 1e12
    # the same launch on the HBM lens: its algorithmic bytes (the complex64
    # factor written once, the scaled complex128 pattern rows and the
    # right-hand side read once) over its time
    alg_bytes = nsys_main * (n * (mb_mixed + 1) * 8.0 + n * 8.0 + n * 16.0)
    hbm_peak, hbm_src = hbm_peak_gbs()
    hbm_ach = alg_bytes / (fac_avg_ms * 1e-3) / 1e9
    hbm_view = {"bound": "hbm", "achieved": hbm_ach, "peak": hbm_peak, "unit": "GB/s", "frac": hbm_ach / hbm_peak,
                "peak_source": hbm_src,
                "algorithmic": "per system: n (mb+1) 8 B of complex64 factor and n 8 B of forward substitution "
                               "written, n 16 B of right-hand side read (the pattern rows' reads excluded)"}
    if bound == "tensor":
        peak, peak_source = tensor_peak_tflops()
    else:
        peak = fp32_sgemm_tflops(stream)
        peak_source = "cuBLAS SGEMM 8192^3, TF32 off, measured in this run (best of 3, CUDA events)"
    traffic = read_profile_traffic(f"{kname}_cfg2.txt")
    line = {
        "metric": METRIC, "value": value, "unit": "units/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 factor + f64 refinement (c128 assembly, residuals, quadrature, J)",
        "data": "synthetic (seeded model and survey with the configuration's shapes)",
        "config": workload_config(args.config, s, K),
        "parallelism": "replicas" if world > 1 else "single GPU",
        "launch": "forward + Jacobian calls" if args.no_graph else
                  "forward + Jacobian as one CUDA graph (crgpu_forward_sens_graph)",
        "refinement": {"maxit": args.refine_maxit, "tol": args.refine_tol, "iterations": statistics.mean(iters)},
        "autotuned_kernels": tune,
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
        "e2e": {"value": 1e3 / e2e_ms, "unit": "units/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "d2h_link_gbs": link_gbs},
        "plain": {"value": 1e3 / plain_ms, "unit": "units/s", "ms_per_step": plain_ms,
                  "ms_factor": plain_stats["ms_factor"], "ms_solve": plain_stats["ms_solve"],
                  "ms_sens": plain_stats["ms_sens"],
                  "roofline": {"kernel": "k_factor_plain_reg", "bound": "fp64",
                               "achieved": flops_factor / (plain_stats["ms_factor"] * 1e-3) / 1e12,
                               "peak": fp64_peak, "unit": "TFLOP/s",
                               "frac": flops_factor / (plain_stats["ms_factor"] * 1e-3) / 1e12 / fp64_peak,
                               "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (best of 3, CUDA events)"}},
        "speedup_mixed_vs_plain": plain_ms / ms_per_step,
        "mixed_vs_plain_rel_err": {"volt": err_v, "jacobian": err_j},
        "accuracy_target": {"volt": 1e-6, "jacobian": 1e-5, "met": bool(err_v < 1e-6 and err_j < 1e-5)},
        "phases_ms": {"factor": fac_avg_ms, "solve": mixed_stats["ms_solve"],
                      "forward": mixed_stats["ms_forward"], "sens": statistics.mean(sens_ms)},
        "factor_band": {"grid_mb": mb, "factored_mb": mb_mixed,
                        "node_order": "geometric" if mb_mixed != mb else "grid"},
        "roofline": {"kernel": kname, "bound": bound, "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_source,
                     "algorithmic": "4*n*mb^2 flops per band system (complex L L^T) at the factored band, "
                                    "the systems of the timed factor launch",
                     "systems": nsys_main,
                     "hbm_view": hbm_view,
                     "note": FACTOR_NOTES.get(kname, "")},
    }
    kwn, kwnwi = mixed.kwn, mixed.kwnwi
    mixed.close()
    if rank == 0 and args.cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(s, kwn, kwnwi)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_ensemble(args):
    """Config 5: 256 independent problems of uneven size (forward + Jacobian
    each), run concurrently on the contexts' streams from a pool of worker
    threads; value = problems per second."""
    import torch

    from titatest_gb300 import MIXED, synth
    from titatest_gb300.ensemble import Ensemble

    torch.cuda.set_device(0)
    probs = synth.config5(count=args.ensemble_count)
    # per-problem tuning is off by default here: choices timed one problem at a
    # time do not maximise the throughput of concurrent problems (measured on
    # config 5: 25.4 problems/s tuned against 27.1 with the built-in choices)
    ens = Ensemble(probs, precision=MIXED, workers=args.workers, refine_maxit=args.refine_maxit,
                   refine_tol=args.refine_tol, autotune=args.autotune_ensemble)
    go = (lambda: ens.run_batched(sens_mode=0)) if args.ensemble_batched else (lambda: ens.run(sens_mode=0))
    for _ in range(max(1, args.warmup)):
        go()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        ev0.record()
        t0 = time.time()
        for _ in range(args.steps):
            go()
        torch.cuda.synchronize()
        wall = time.time() - t0
        ev1.record()
        torch.cuda.synchronize()
    ms = wall * 1e3 / args.steps
    line = {
        "metric": "config-5 ensemble: forward+Jacobian problems/s (complex64 + FP64 refinement)",
        "value": len(probs) * 1e3 / ms, "unit": "problems/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 factor + f64 refinement",
        "data": "synthetic (seeded meshes 40x15..300x80 quads, 24-128 electrodes, 200-6000 quadrupoles)",
        "config": {"workload": f"config5: {len(probs)} problems, {sum(p.grid.sanz for p in probs)} nodes in total",
                   "workers": args.workers,
                   "parallelism": ("single GPU, waves of problems: one tensor-core factor launch over all "
                                   "systems of a wave, the other steps on the problems' streams" if args.ensemble_batched
                                   else "single GPU, one context per problem on concurrent streams"),
                   "band_order": "geometric node order for mixed bands beyond the tensor-core window"},
        "clocks": clk.summary(),
    }
    print(json.dumps(line))
    return 0


def run_inversion(args):
    """Config 4: the CRTomo Gauss-Newton complex inversion (structured
    smoothness, lambda search) of synthetic data on the 400x100-quad,
    192-electrode, 20000-quadrupole mesh: 8 iterations, CG capped at 100
    steps, mixed precision.  value = seconds per GN iteration (all its lambda
    and step trials: forward, Jacobian, update); RMS per iteration."""
    import torch

    from titatest_gb300 import MIXED, synth
    from titatest_gb300 import inversion as I
    from titatest_gb300.crmod import rwaven

    torch.cuda.set_device(0)
    s = synth.config4()
    g, sv = s.grid, s.survey
    kwn, kwnwi = rwaven(g, sv)
    b = I.DeviceBackend(g, sv, kwn, kwnwi, 1, False, 0, MIXED, refinement=(args.refine_maxit, args.refine_tol))
    try:
        # data: the true model's response with 3% + 1e-4 ohm and 1 mrad noise
        t0 = time.perf_counter()
        V = np.exp(-b.forward(s.sigma))
        t_first = time.perf_counter() - t0
        rng = np.random.default_rng(4001)
        bet, pha = np.abs(V), np.angle(V) * 1e3
        noisy = bet + (0.03 * bet + 1e-4) * rng.standard_normal(len(bet))
        while np.any(noisy <= 0):  # redraw the noise of a datum that would change sign
            bad = noisy <= 0
            noisy[bad] = bet[bad] + (0.03 * bet[bad] + 1e-4) * rng.standard_normal(int(bad.sum()))
        pha_n = pha + rng.standard_normal(len(pha))
        cfg = I.CRTomoConfig(mswitch=0, delem="", delectr="", dstrom="", ramd="", ldiff=False, dd0="", dm0="",
                             dfm0="", nx=400, nz=100, alfx=1.0, alfz=1.0, itmax=8, ldc=False, lrobust=False,
                             lfphai=False, stabw0=3.0, stabm0=1e-4, stabpA1=0.0, stabpB=0.0, stabpA2=0.0,
                             stabp0=1.0, lrho0=True, bet0=100.0, pha0=-10.0, lagain=False, swrtr=1, lsink=False,
                             nsink=0, lrandb2=False, drandb="", ltri=0)
        data = I.make_data(sv.strnr, sv.vnr, noisy, pha_n, cfg)
        inv = I.Inversion(g, data, cfg, b, ncgmax=100)
        calls = {"forward": 0, "sens": 0, "update": 0}
        times = {"forward": 0.0, "sens": 0.0, "update": 0.0}

        def timed(name, fn):
            def w(*a, **k):
                t = time.perf_counter()
                r = fn(*a, **k)
                times[name] += time.perf_counter() - t
                calls[name] += 1
                return r
            return w

        b.forward = timed("forward", b.forward)
        b.sensitivities = timed("sens", b.sensitivities)
        b.update = timed("update", b.update)
        torch.cuda.synchronize()
        with ClockSampler(0) as clk:
            t0 = time.perf_counter()
            rows = inv.run()
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
    finally:
        b.close()
    cpu = None
    if args.cpu_baseline:
        # the oracle on one whole forward + Jacobian unit, multiplied by the
        # forwards and Jacobians of one GN iteration as this run made them
        # (the CPU CG is not included)
        cb = cpu_baseline(s, kwn, kwnwi)
        n_it_ = max(1, sum(1 for r in rows if r.kind == "IT") - 1)
        est = (calls["forward"] * cb["forward_s"] + calls["sens"] * cb["sens_s"]) / n_it_
        cpu = {"value": est, "unit": "s/iteration (forwards + Jacobians only)", "cores": cb["cores"],
               "kind": "port", "sample": cb["sample"], "forward_s": cb["forward_s"], "sens_s": cb["sens_s"]}
    its = [r for r in rows if r.kind == "IT"]
    n_it = max(1, len(its) - 1)
    line = {
        "metric": "config-4 CRTomo Gauss-Newton complex inversion: seconds per GN iteration (mixed precision)",
        "value": wall / n_it, "unit": "s/iteration", "n_gpus": 1, "steps": n_it, "warmup": 0,
        "ms_per_step": wall * 1e3 / n_it, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 factor + f64 refinement; f64 Jacobian products and CG",
        "data": "synthetic (config-4 model, its response with 3% + 1e-4 ohm and 1 mrad noise)",
        "config": {"workload": workload_string(4, s, len(kwn)) + ", 8 GN iterations, CG <= 100 steps",
                   "regularisation": "structured smoothness (ltri 0, 400 x 100), lambda search of src/inv.f90",
                   "parallelism": "single GPU"},
        "rms_per_iteration": [round(r.nrmsd, 4) for r in its], "lambda_per_iteration": [r.lam for r in its[1:]],
        "status": inv.status, "trials": len(rows) - len(its), "calls": calls,
        "seconds": {k: round(v, 3) for k, v in times.items()}, "first_forward_s": round(t_first, 3),
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    return 0


def run_case(args):
    """--case: one forward (and optionally the Jacobian, an update, the model
    uncertainty) of a configuration, printed as plain timings: the command
    that the ncu captures in profiles/ run.  --batch limits the systems per
    factor batch, so that a capture holds one launch of known size."""
    from titatest_gb300 import MIXED, PLAIN, CRMod, synth

    s = synth.make(args.config)
    prec = MIXED if args.precision == "mixed" else PLAIN
    with CRMod(s.grid, s.survey, precision=prec, band_order=args.band_order) as m:
        m.set_refinement(args.refine_maxit, args.refine_tol)
        if args.autotune_case:
            print("tune", m.autotune(s.sigma), flush=True)
        if args.batch:
            g = s.grid
            esz = 8 if prec == MIXED else 16
            mbf = factored_band(m, g)
            per = g.sanz * (mbf + 1) * esz + (g.sanz * 12 * 16) + g.sanz * 8 + g.sanz * (3 * 16 + esz) + 64
            m.set_memory_budget(int(per * args.batch + per // 2))
        for _ in range(args.repeat):
            t = time.time()
            out = m.forward(s.sigma)
            st = m.stats()
            msg = (f"forward {1e3 * (time.time() - t):.1f} ms, batches {st['nbatches']}, factor "
                   f"{st['ms_factor']:.1f} ms, solve {st['ms_solve']:.1f} ms, refinement {st['refine_iterations']}")
            if args.sens:
                J = m.sens(0)
                msg += f", sens {m.stats()['ms_sens']:.1f} ms, |J|max {np.abs(J).max():.3e}"
            print(msg, flush=True)
        assert np.all(np.isfinite(out["volt"]))
        if args.update_steps:
            from titatest_gb300 import regularization as R
            sa = m.forward(s.sigma, volt_mode=1)["sigmaa"]
            m.sens_on_device(1)
            dat = sa - np.log(1.03)
            w = np.full(len(sa), 1.0 / 0.03 ** 2)
            sm = R.bsmatmreg(s.grid, s.nx, s.nz)
            t = time.time()
            _, dpar, _, _, ncg = m.update(w, np.ones(len(sa), np.int32), dat, sa, 0, sm, nx=s.nx, lam=300.0,
                                          eps=1e-4, ncgmax=args.update_steps, par=np.log(s.sigma))
            print(f"update {1e3 * (time.time() - t):.1f} ms, {ncg} CG steps, |dpar|max {np.abs(dpar).max():.3e}",
                  flush=True)
            if args.mcm:
                t = time.time()
                d = m.mcm(w, np.ones(len(sa), np.int32), 0, sm, nx=s.nx, lam=300.0)
                print(f"mcm {1e3 * (time.time() - t):.1f} ms for manz {len(d['cov1'])} (ata, ata_reg, Cholesky "
                      f"inverse, resolution, cov2), min cov1 {d['cov1'].min():.3e}", flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=2)
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--refine-maxit", type=int, default=8)
    ap.add_argument("--no-autotune", action="store_true", help="keep the built-in kernel choices")
    ap.add_argument("--no-graph", action="store_true",
                    help="time the forward and Jacobian calls instead of their CUDA-graph replay")
    ap.add_argument("--autotune-ensemble", action="store_true", help="config 5: autotune every problem shape")
    ap.add_argument("--refine-tol", type=float, default=None,
                    help="mixed refinement stop: max|dx| <= tol max|x|.  Default 0.1 on config 2 (one "
                         "correction: volt within 1.4e-7 and J within 9e-7 of complex128, against the targets "
                         "1e-6 / 1e-5; both errors are measured and checked in every line), 1e-2 elsewhere")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--workers", type=int, default=8, help="config 5: concurrent worker streams")
    ap.add_argument("--ensemble-batched", action="store_true",
                    help="config 5: waves of problems with one factor launch each (crgpu_forward_sens_batch) "
                         "instead of one context per problem on worker streams")
    ap.add_argument("--ensemble-count", type=int, default=256, help="config 5: number of problems")
    ap.add_argument("--case", action="store_true",
                    help="plain timings of one forward of --config (the command the ncu captures run)")
    ap.add_argument("--precision", choices=["mixed", "plain"], default="mixed", help="--case: precision")
    ap.add_argument("--band-order", type=int, default=1, choices=[0, 1, 2],
                    help="crgpu_create2 band order: 0 the grid's band, 1 geometric for mixed bands beyond the "
                         "tensor-core window, 2 geometric whenever narrower")
    ap.add_argument("--autotune-case", action="store_true", help="--case: autotune the factor kernel first")
    ap.add_argument("--batch", type=int, default=0, help="--case: systems per factor batch (0: as many as fit)")
    ap.add_argument("--repeat", type=int, default=1, help="--case: forwards to run")
    ap.add_argument("--sens", action="store_true", help="--case: also the Jacobian")
    ap.add_argument("--update-steps", type=int, default=0,
                    help="--case: also the CRTomo Jacobian and one update with at most this many CG steps")
    ap.add_argument("--mcm", action="store_true", help="--case with --update-steps: also crgpu_mcm")
    args = ap.parse_args()
    if args.refine_tol is None:
        args.refine_tol = 1e-8 if args.case else 0.1 if args.config == 2 else 1e-2
    if args.case:
        return run_case(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.config == 5:
        return run_ensemble(args)
    if args.config == 4:
        return run_inversion(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
