"""Benchmark: 2.5D complex-resistivity forward + Jacobian units per second.

One unit (a "step") is the complete forward -- every wavenumber x current
electrode assembled, factorised and solved, back-transformed, voltages -- plus
the full Jacobian (src/bsens.f90), for one conductivity model.  The workload
is the 200x60-quad, 96-electrode, 4000-quadrupole configuration (synthetic,
seeded; titatest_gb300.synth.config2).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

value : mixed mode (complex64 factor + FP64 refinement), inputs resident on
        the device, timed with CUDA events on the library's stream;
e2e   : the same unit through the host C ABI (crgpu_forward + crgpu_sens with
        pinned host buffers: sigma in, voltages and the Jacobian out), with
        d2h_link_gbs, the rate of a plain pinned copy of the Jacobian's bytes
        in the same run (the host link is shared and its rate varies);
plain : the complex128 mode on the same inputs (the reference arithmetic),
        with the mixed/plain speed-up and the error of mixed against plain.
--impl reference times the oracle (the plain-C restatement of the reference
routines, OpenMP over all host cores) on a bounded sample of the same unit.
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
# CPU baseline: the oracle (plain-C restatement, OpenMP) on a bounded sample
# ---------------------------------------------------------------------------
def cpu_baseline(s, kwn, kwnwi, kpot, target_s=12.0, threads=None):
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    P = O.Problem(s.grid, s.survey)
    K, E = len(kwn), s.survey.eanz
    nsys = K * E
    rng = np.random.default_rng(7)
    # set-up (precal for all wavenumbers and electrodes) is timed once; then
    # systems are solved in parallel (one per thread), as many rounds as fit
    t0 = time.perf_counter()
    P.forward_pairs(s.sigma, kwn, kwnwi, np.zeros((0, 2), np.int32), nthreads=threads)
    t_setup = time.perf_counter() - t0
    pairs_all = np.array([(k, l) for k in range(K) for l in range(E)], np.int32)
    nsample = 2 * threads
    t_fwd = 0.0
    solved = 0
    while t_fwd < target_s * 0.6 and solved < nsys:
        pick = pairs_all[rng.choice(nsys, size=min(nsample, nsys), replace=False)]
        t0 = time.perf_counter()
        P.forward_pairs(s.sigma, kwn, kwnwi, pick, nthreads=threads)
        t_fwd += time.perf_counter() - t0 - t_setup
        solved += len(pick)
    fwd_per_unit = t_setup + t_fwd / solved * nsys
    # Jacobian: a sample of measurements (timing only; the numbers are those
    # of the GPU kpot)
    from titatest_gb300 import formats as F
    q = max(threads * 4, 64)
    idx = rng.choice(s.survey.nanz, size=min(q, s.survey.nanz), replace=False)
    sub = F.Survey(enr=s.survey.enr, strnr=s.survey.strnr[idx], vnr=s.survey.vnr[idx],
                   strom=s.survey.strom[idx])
    Ps = O.Problem(s.grid, sub)
    t0 = time.perf_counter()
    Ps.bsens(kpot, kwn, kwnwi, s.sigma, None, mode=0, nthreads=threads)
    t_j = time.perf_counter() - t0
    sens_per_unit = t_j / len(idx) * s.survey.nanz
    unit_s = fwd_per_unit + sens_per_unit
    return {"value": 1.0 / unit_s, "unit": "units/s", "cores": threads, "kind": "port",
            "sample": (f"{solved} of {nsys} (k,l) systems and {len(idx)} of {s.survey.nanz} Jacobian rows, "
                       f"scaled to one unit ({t_fwd + t_j:.1f} s of CPU work)"),
            "seconds_per_unit": unit_s, "forward_s": fwd_per_unit, "sens_s": sens_per_unit}


def workload_string(cfg: int, s, K: int) -> str:
    g, sv = s.grid, s.survey
    kind = "triangles" if getattr(s, "triangles", False) else "quads"
    nsys = K * sv.eanz
    return (f"config{cfg}: {g.elanz} {kind}, {g.sanz} nodes, mb={g.mb}, {sv.eanz} electrodes, "
            f"{sv.nanz} quadrupoles, {K} wavenumbers ({nsys} band systems)")


def run_reference(args):
    rank, world, _ = _dist_env()
    if rank != 0:
        return 0
    from titatest_gb300 import synth
    from oracle import oracle as O
    s = synth.make(args.config)
    P = O.Problem(s.grid, s.survey)
    kwn, kwnwi = P.rwaven()
    # potentials for the Jacobian timing: zeros have the same cost
    kpot = np.zeros((len(kwn), s.survey.eanz, s.grid.sanz), np.complex128)
    vals = []
    for it in range(args.warmup + args.steps):
        cb = cpu_baseline(s, kwn, kwnwi, kpot, target_s=args.ref_seconds)
        if it >= args.warmup:
            vals.append(cb["value"])
    v = statistics.median(vals)
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "units/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (seeded)",
            "config": {"workload": workload_string(args.config, s, len(kwn)),
                       "parallelism": f"OpenMP {cb['cores']} threads"},
            "cpu_baseline": cb,
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

    mixed = CRMod(g, sv, precision=MIXED)
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
    plain = CRMod(g, sv, precision=PLAIN)
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

    # ---- roofline of the dominant kernel (the complex64 band factorisation on
    #      the tensor cores); algorithmic work = complex L L^T of every system
    n, mb = g.sanz, g.mb
    nsys = K * sv.eanz
    flops_factor = nsys * 4.0 * n * mb * mb  # 8 flops per complex multiply-add, n*mb^2/2 of them
    fac_avg_ms = statistics.mean(fac_ms)
    achieved = flops_factor / (fac_avg_ms * 1e-3) / 1e12
    peak, peak_source = tensor_peak_tflops()
    traffic = read_profile_traffic("k_factor_tc_cfg2.txt")
    line = {
        "metric": METRIC, "value": value, "unit": "units/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 factor + f64 refinement (c128 assembly, residuals, quadrature, J)",
        "data": "synthetic (seeded model and survey with the configuration's shapes)",
        "config": {"workload": workload_string(args.config, s, K),
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "launch": "forward + Jacobian calls" if args.no_graph else
                             "forward + Jacobian as one CUDA graph (crgpu_forward_sens_graph)",
                   "l2": "inputs larger than L2 (band factors of all systems, ~%d GB)" % int(
                       nsys * n * (mb + 1) * 8 / 1e9),
                   "refinement": {"maxit": args.refine_maxit, "tol": args.refine_tol,
                                  "iterations": statistics.mean(iters)},
                   "autotuned_kernels": tune},
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
        "e2e": {"value": 1e3 / e2e_ms, "unit": "units/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "d2h_link_gbs": link_gbs},
        "plain": {"value": 1e3 / plain_ms, "unit": "units/s", "ms_per_step": plain_ms,
                  "ms_factor": plain_stats["ms_factor"], "ms_solve": plain_stats["ms_solve"],
                  "ms_sens": plain_stats["ms_sens"]},
        "speedup_mixed_vs_plain": plain_ms / ms_per_step,
        "mixed_vs_plain_rel_err": {"volt": err_v, "jacobian": err_j},
        "accuracy_target": {"volt": 1e-6, "jacobian": 1e-5, "met": bool(err_v < 1e-6 and err_j < 1e-5)},
        "phases_ms": {"factor": fac_avg_ms, "solve": mixed_stats["ms_solve"],
                      "forward": mixed_stats["ms_forward"], "sens": statistics.mean(sens_ms)},
        "roofline": {"kernel": "k_factor_tc", "bound": "tensor", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_source,
                     "algorithmic": "4*n*mb^2 flops per band system (complex L L^T), all systems of one forward",
                     "note": "latency-bound band factor: each 4-column step is a serial panel plus 4 tf32 MMAs "
                             "(3 hi/lo products + row injection) on a 128x128 complex window"},
    }
    if rank == 0 and args.cpu_baseline:
        kpot = mixed.forward(s.sigma, kpot=True)["kpot"]
        line["cpu_baseline"] = cpu_baseline(s, mixed.kwn, mixed.kwnwi, kpot, target_s=args.ref_seconds)
    mixed.close()
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_ensemble(args):
    """Config 5: 256 independent problems of uneven size (forward + Jacobian
    each), run concurrently on worker streams; value = problems per second."""
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
    for _ in range(max(1, args.warmup)):
        ens.run(sens_mode=0)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        ev0.record()
        t0 = time.time()
        for _ in range(args.steps):
            ens.run(sens_mode=0)
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
                   "workers": args.workers, "parallelism": "single GPU, concurrent streams"},
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
        kpot = b.m.forward(s.sigma, kpot=True)["kpot"] if args.cpu_baseline else None
    finally:
        b.close()
    cpu = None
    if kpot is not None:
        # the oracle on a bounded sample of the forward's systems and of the
        # Jacobian's rows, scaled to the forwards and Jacobians of one GN
        # iteration as this run made them (the CPU CG is not included)
        cb = cpu_baseline(s, kwn, kwnwi, kpot, target_s=args.ref_seconds)
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
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--workers", type=int, default=8, help="config 5: concurrent worker streams")
    ap.add_argument("--ensemble-count", type=int, default=256, help="config 5: number of problems")
    args = ap.parse_args()
    if args.refine_tol is None:
        args.refine_tol = 0.1 if args.config == 2 else 1e-2
    if args.impl == "reference":
        return run_reference(args)
    if args.config == 5:
        return run_ensemble(args)
    if args.config == 4:
        return run_inversion(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
