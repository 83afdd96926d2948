#!/usr/bin/env python
"""Benchmark of the LASSIE GB300 integrator on the batched workload.

Workload: 2048 independent mass-action instances (species N_i ~ U{32..512},
R_i = N_i, 1-2 reactant structure, k ~ 10^U(-4,4), t in [0,20], 50 samples),
integrated with the reference's step control (RKF45, stiffness switch,
backward-Euler modified Newton) by the mixed-precision batched form (FP32 LU,
FP64 refinement) in one persistent launch.  A step integrates the whole
batch; ``value`` is instances per second with inputs resident in HBM,
``e2e`` the same through the public host-buffer API (``lassie_solve_batch``).

Under the reference's step control a few instances never finish in practice:
every NaN/negative revert divides the backward-Euler step by 10 for good, so
22 of the 2048 end at dt = 1e-4 (2e5 steps), one at 1e-6 (2e7 steps), and one
cycles through RKF45 retries whose step grows after each positivity reject.
Every instance therefore gets the same cap of loop iterations (--max-steps,
default 25000: the instances whose step ends at 1e-3 need about 20000);
``value`` counts only instances that reached the end of the horizon, and the
capped ones are reported.

Extra keys: the plain FP64 GPU form and the max relative error against it on
a sample, the mixed-vs-FP64 parity per configuration, the adjoint, the
batched RHS and Newton-matrix kernels' HBM bandwidth, the BDF controller on
the same batch (both forms), the roofline of the integrator kernel, the CPU
baselines (the oracle port, and scipy LSODA, on the host cores), the SM clocks
sampled during the timed region.

``--impl reference`` times the reference algorithm's CPU implementation (the
oracle port, all host threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "sims/s and adjoint grads/s at rtol 1e-6 vs plain FP64 GPU form; RHS HBM GB/s"
WORKLOAD = "c4: 2048 instances, N_i~U{32..512}, R_i=N_i, k~10^U(-4,4), t in [0,20], 50 samples"
RTOL, ATOL = 1e-6, 1e-9


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def load_traffic(alg_flops):
    """DRAM bytes of one integrator launch: the bytes per algorithmic FLOP of
    a committed ncu capture of the kernel on a small case
    (profiles/compat_kernel_traffic.json), times this launch's algorithmic
    FLOPs -- the kernel's traffic grows with its factorisations and sweeps.
    None without the file."""
    p = os.path.join(ROOT, "profiles", "compat_kernel_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        per_flop = json.load(f).get("dram_bytes_per_algorithmic_flop")
    return None if per_flop is None else per_flop * alg_flops


def spread_classes(mixed, fp64, mixed_stats, cap):
    """Instances of the FP64-vs-mixed sample by the oracle's own spread
    (tests/oracle_fixtures/c4_spread.npz, the same 152 instances on t in
    [0, 2]): within rtol 1e-6 / atol 1e-9 of the FP64 form (which equals the
    oracle bit for bit) before the spread's first divergence and within twice
    its excess after it -- the FP64 solvers' spread first, else the normwise
    one -- or outside both.  None without the fixture or for another sample."""
    p = os.path.join(ROOT, "tests", "oracle_fixtures", "c4_spread.npz")
    if not os.path.exists(p):
        return None
    f = np.load(p)
    if len(f["index"]) != len(mixed) or int(f["cap"]) != cap:
        return None
    out = {"fp64_solvers": 0, "normwise_solvers": 0, "outside": 0, "capped_in_oracle": 0}
    for j, (a, b, st) in enumerate(zip(mixed, fp64, mixed_stats)):
        if int(f["status"][j]) != 0:
            out["capped_in_oracle"] += 1
            continue
        e = np.max(np.abs(a - b) - 1e-9 - 1e-6 * np.abs(b), axis=1)

        def within(first, worst):
            return st["status"] == 0 and np.all(e[:first] <= 0) and e.max() <= 2 * worst

        if within(int(f["first_divergence"][j]), float(f["worst_excess"][j])):
            out["fp64_solvers"] += 1
        elif ("first_divergence_normwise" in f.files and
              within(int(f["first_divergence_normwise"][j]), float(f["worst_excess_normwise"][j]))):
            out["normwise_solvers"] += 1
        else:
            out["outside"] += 1
    return out


def pipe_work(stats, models):
    """Work of the mixed batched integrator on the pipes that bound it.
    FP32 (the FMA pipes): the Gauss-Jordan inverses, 2 N^3 per factorisation,
    and the refinement's matrix-vector products, 2 N^2 per sweep.  FP64: one
    RHS evaluation costs about nnz_A + 2 nnz_H operations (products of the
    reactant powers, then the signed species sums) -- six per RKF45 attempt
    and one per Newton iteration -- and one refinement residual about the
    same through J v plus 3 N."""
    f32 = f64 = 0.0
    for s, m in zip(stats, models):
        n = float(m.n_species)
        na = float(np.count_nonzero(m.left))
        nh = float(np.count_nonzero(np.asarray(m.right) - np.asarray(m.left)))
        f32 += s["lu_factorisations"] * 2.0 * n ** 3 + s["refine_sweeps"] * 2.0 * n * n
        attempts = s["rkf_accepts"] + s["rkf_retries"] + s["be_steps"]
        f64 += (6.0 * attempts + s["newton_iters"]) * (na + 2.0 * nh)
        f64 += s["refine_sweeps"] * (na + 2.0 * nh + 3.0 * n)
    return f32, f64


def lu_flops(stats, models, engine):
    """Algorithmic FLOPs of the dense linear algebra the integration did:
    (2/3)N^3 per factorisation + 2N^2 per solve (an LU's triangular-solve
    pair).  The mixed form's Gauss-Jordan inverse does 2N^3 per
    factorisation; the roofline counts the LU's algorithmic figure."""
    tot = 0.0
    for s, m in zip(stats, models):
        n = float(m.n_species)
        pairs = s["refine_sweeps"] if engine == "mixed" else s["newton_iters"]
        tot += s["lu_factorisations"] * (2.0 / 3.0) * n ** 3 + pairs * 2.0 * n * n
    return tot


def max_rel_err(a_list, b_list):
    import numpy as np
    worst, bad = 0.0, 0
    for a, b in zip(a_list, b_list):
        d = np.abs(a - b)
        rel = d / np.maximum(np.abs(b), ATOL / RTOL)
        worst = max(worst, float(rel.max()) if rel.size else 0.0)
        bad += int(np.count_nonzero(d > ATOL + RTOL * np.abs(b)))
    return worst, bad


# The CPU sample, the same for the reference arm and the cpu_baseline key:
# every 128th instance of the workload (16 instances, one per host core of
# the GPU machine) on the first 5 % of its horizon, loop-iteration cap scaled
# alike; sims/s extrapolated to the whole horizon.  `--cpu-full-horizon`
# runs the same 16 instances over the whole horizon once, which is how the
# extrapolation is checked.
CPU_STRIDE, CPU_T_FRAC = 128, 0.05


def cpu_sample_models(n_total, t_frac=CPU_T_FRAC, stride=CPU_STRIDE):
    from lassie_gb300 import synth
    idx = list(range(0, n_total, stride))
    if t_frac >= 1.0:
        return [synth.make_c4_instance(q) for q in idx]
    return [synth.shorten(synth.make_c4_instance(q), 20.0 * t_frac,
                          max(2, int(round(50 * t_frac))))
            for q in idx]


def flush_host_caches(buf=[]):
    """Write 256 MB of host memory (more than the host's caches) before a
    timed CPU step, as the GPU arm flushes its L2."""
    import numpy as np
    if not buf:
        buf.append(np.empty(256 * 1024 * 1024 // 8))
    buf[0].fill(1.0)


def cpu_baseline(n_total, threads=None, stride=CPU_STRIDE, t_frac=CPU_T_FRAC, max_steps=25000):
    """The oracle port (the reference algorithm) on the host cores: every
    `stride`-th instance of the workload on the first `t_frac` of its horizon
    (loop-iteration cap scaled alike), extrapolated to the horizon; completed
    instances only."""
    from oracle import oracle as O
    models = cpu_sample_models(n_total, t_frac, stride)
    threads = threads or os.cpu_count() or 1
    frac = min(1.0, t_frac)
    flush_host_caches()
    t0 = time.perf_counter()
    _, stats, status = O.solve_batch(models, threads=threads,
                                     max_steps=max(1, int(max_steps * frac)))
    dt = time.perf_counter() - t0
    done = sum(1 for s in status if s == 0)
    sims = done / (dt / frac)
    return {"value": sims, "unit": "sims/s", "cores": threads, "kind": "port",
            "sample": f"{len(models)} of the {n_total} instances (every {stride}th, "
                      f"{done} completed), t in [0,{20.0 * frac:g}] (= {frac:g} of the "
                      f"horizon), time scaled by {1 / frac:g}; {dt:.2f} s wall",
            "seconds": dt, "be_steps": sum(st["be_steps"] for st in stats),
            "capped": sum(1 for s in status if s != 0)}


def run_cpu_full_horizon(args):
    """The CPU sample over the whole horizon next to its extrapolated
    short-horizon figure (one JSON line; tens of minutes)."""
    short = cpu_baseline(args.instances, max_steps=args.max_steps)
    full = cpu_baseline(args.instances, t_frac=1.0, max_steps=args.max_steps)
    print(json.dumps({"cpu_sample_extrapolated": short, "cpu_sample_full_horizon": full,
                      "full_over_extrapolated": full["value"] / short["value"]}), flush=True)
    return 0


def _lsoda_one(q):
    """One workload instance with scipy's LSODA (odeint): the oracle's RHS and
    exact dense Jacobian through ctypes, rtol 1e-6, atol 1e-12, mxstep 10000.
    Returns (seconds, success)."""
    import warnings
    from scipy.integrate import odeint
    from lassie_gb300 import synth
    from oracle import oracle as O
    m = synth.make_c4_instance(q)
    om = O.OracleModel(m.left, m.right)
    k = m.k
    t0 = time.perf_counter()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        _, info = odeint(lambda x, t: om.rhs(k, x), m.x0, m.t,
                         Dfun=lambda x, t: om.jacobian_exact(k, x), rtol=1e-6, atol=1e-12,
                         mxstep=10000, full_output=True)
    return time.perf_counter() - t0, info.get("message", "") == "Integration successful."


def lsoda_baseline(n_total, stride=128, threads=None):
    """The CPU baseline the hot-path table defines: scipy's LSODA with the
    analytic Jacobian on the host cores (one process per core, spawn-started),
    on every `stride`-th instance of the workload over its whole horizon.  A
    different algorithm from the reference's loop (error control), so it is
    the CPU counterpart of the BDF controller."""
    import multiprocessing as mp
    idx = list(range(0, n_total, stride))
    threads = threads or os.cpu_count() or 1
    # one BLAS/OpenMP thread per worker process (the workers inherit the
    # environment at spawn); otherwise every worker's BLAS pool spans all cores
    # and LSODA's many small BLAS calls slow down by orders of magnitude
    pinned = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {v: os.environ.get(v) for v in pinned}
    for v in pinned:
        os.environ[v] = "1"
    try:
        t0 = time.perf_counter()
        with mp.get_context("spawn").Pool(min(threads, len(idx))) as pool:
            res = pool.map(_lsoda_one, idx)
        dt = time.perf_counter() - t0
    finally:
        for v, val in saved.items():
            if val is None:
                os.environ.pop(v, None)
            else:
                os.environ[v] = val
    done = sum(1 for _, ok in res if ok)
    return {"value": done / dt, "unit": "sims/s", "cores": min(threads, len(idx)),
            "kind": "scipy LSODA (odeint, analytic Jacobian, rtol 1e-6, atol 1e-12)",
            "sample": f"{len(idx)} of the {n_total} instances (every {stride}th), full "
                      f"horizon t in [0,20]; {done} integrated successfully; {dt:.2f} s wall",
            "cpu_seconds_per_instance": sum(t for t, _ in res) / len(res)}


def _lsoda_c3_child(t_reached, cap_s):
    """Child process of lsoda_c3: odeint interval by interval over the C3
    sample times, publishing the time reached after each interval."""
    import warnings
    from scipy.integrate import odeint
    from lassie_gb300 import synth
    from oracle import oracle as O
    m = synth.make_c3()
    om = O.OracleModel(m.left, m.right)
    x = m.x0.copy()
    t0 = time.perf_counter()
    for i in range(1, len(m.t)):
        if time.perf_counter() - t0 > cap_s:
            return
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            ys = odeint(lambda y, t: om.rhs(m.k, y), x, [m.t[i - 1], m.t[i]],
                        Dfun=lambda y, t: om.jacobian_exact(m.k, y), rtol=1e-6, atol=1e-12,
                        mxstep=10000)
        x = ys[-1]
        t_reached.value = float(m.t[i])


def lsoda_c3(cap_s=120.0):
    """The CPU baseline's C3 figure: scipy LSODA (odeint, analytic dense
    4096 x 4096 Jacobian, rtol 1e-6, atol 1e-12) on one core, stopped at a
    wall-clock cap (a spawned child, ended by its own PID when an interval
    outlasts the cap).  Reports how far it got."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    reached = ctx.Value("d", 0.0)
    p = ctx.Process(target=_lsoda_c3_child, args=(reached, cap_s))
    t0 = time.perf_counter()
    p.start()
    p.join(cap_s + 30.0)
    if p.is_alive():
        p.terminate()
        p.join()
    wall = time.perf_counter() - t0
    t_end = 50.0
    return {"kind": "scipy LSODA (odeint, analytic dense Jacobian, rtol 1e-6, atol 1e-12), "
                    "one core", "cap_s": cap_s, "t_reached": reached.value, "t_end": t_end,
            "capped": reached.value < t_end, "seconds": wall,
            "sims_per_s_extrapolated": (reached.value / t_end) / wall if reached.value > 0 else 0.0}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    for _ in range(args.warmup):
        cpu_baseline(args.instances, max_steps=args.max_steps)
    vals, secs = [], []
    for _ in range(args.steps):
        cb = cpu_baseline(args.instances, max_steps=args.max_steps)
        vals.append(cb["value"])
        secs.append(cb["seconds"])
    v = statistics.mean(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "sims/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * statistics.mean(secs), "higher_is_better": True,
        "scaling": args.scaling, "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args),
        "form": "reference algorithm, CPU (oracle port)",
        "cpu_baseline": {"value": v, "unit": "sims/s", "cores": cb["cores"], "kind": "port",
                         "sample": cb["sample"]},
        "e2e": {"value": v, "unit": "sims/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(args):
    """The `config` of both arms' lines: the workload and its loop cap."""
    full = args.instances == 2048 and args.horizon == 20.0
    return {"workload": WORKLOAD if full else
            f"{WORKLOAD} -- reduced: {args.instances} instances, t in [0,{args.horizon:g}]",
            "max_steps_per_instance": args.max_steps,
            "l2": "flushed between steps (256 MB write)"}


def rhs_bandwidth(torch, stream, n_inst=65536, reps=20, warm=3):
    """Batched RHS kernel on one 256-species network with n_inst
    parameterisations (x, k, dx each n_inst*256 doubles, larger than L2)."""
    import ctypes as C
    import numpy as np
    from lassie_gb300 import synth, _native as nat
    from lassie_gb300.solver import NativeModel
    base, _ = synth.make_c5(1)
    m = base[0]
    nm = NativeModel.of(m)
    N, R = m.n_species, m.n_reactions
    dev = torch.device("cuda")
    g = torch.Generator(device=dev).manual_seed(0)
    x = torch.rand((n_inst, N), dtype=torch.float64, device=dev, generator=g)
    k = torch.rand((n_inst, R), dtype=torch.float64, device=dev, generator=g)
    dx = torch.empty_like(x)
    L = nat.load()
    launch = lambda: nat.check(L.lassie_rhs_device(nm.handle, n_inst, k.data_ptr(), x.data_ptr(),  # noqa: E731
                                                   dx.data_ptr(), C.c_void_p(stream.cuda_stream)),
                               "lassie_rhs_device")
    with torch.cuda.stream(stream):
        for _ in range(warm):
            launch()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            launch()
        e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    n_a, n_h = nm.info()[2], nm.info()[3]
    alg = n_inst * (8 * R + 8 * N + 8 * N) + 4 * (R + 1 + n_a + N + 1 + n_h)
    return {"gbs": alg / (ms * 1e-3) / 1e9, "ms_per_launch": ms, "bytes_per_launch": alg,
            "network": "256 species x 256 reactions", "instances": n_inst}


def newton_bandwidth(torch, stream, precision, n_inst=2048, reps=10, warm=3):
    """Batched Newton-matrix kernel (I - h*J(x_b), dense row-major) on one
    256-species network with n_inst parameterisations: 2048 x 256 x 256
    outputs, 1.07 GB in FP64 or 0.54 GB in FP32 per launch (larger than L2).
    Algorithmic bytes: the matrices written plus x and k read."""
    import ctypes as C
    from lassie_gb300 import synth, _native as nat
    from lassie_gb300.solver import NativeModel
    base, _ = synth.make_c5(1)
    m = base[0]
    nm = NativeModel.of(m)
    N, R = m.n_species, m.n_reactions
    dev = torch.device("cuda")
    g = torch.Generator(device=dev).manual_seed(1)
    x = torch.rand((n_inst, N), dtype=torch.float64, device=dev, generator=g)
    k = torch.rand((n_inst, R), dtype=torch.float64, device=dev, generator=g)
    es = 8 if precision == 0 else 4
    M = torch.empty((n_inst, N, N), dtype=torch.float64 if es == 8 else torch.float32, device=dev)
    L = nat.load()
    launch = lambda: nat.check(L.lassie_newton_matrix_device(  # noqa: E731
        nm.handle, n_inst, 0.01, k.data_ptr(), x.data_ptr(), M.data_ptr(), precision,
        C.c_void_p(stream.cuda_stream)), "lassie_newton_matrix_device")
    with torch.cuda.stream(stream):
        for _ in range(warm):
            launch()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            launch()
        e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    # the write-only ceiling on the same buffer: torch's fill kernel
    with torch.cuda.stream(stream):
        for _ in range(warm):
            M.fill_(0.5)
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        f0.record(stream)
        for _ in range(reps):
            M.fill_(0.5)
        f1.record(stream)
    torch.cuda.synchronize()
    fill_gbs = M.numel() * es / (f0.elapsed_time(f1) / reps * 1e-3) / 1e9
    nnz = C.c_int64(0)
    nat.check(L.lassie_jacobian_nnz(nm.handle, C.byref(nnz)), "lassie_jacobian_nnz")
    alg = n_inst * (es * N * N + 8 * (N + R))
    return {"gbs": alg / (ms * 1e-3) / 1e9, "ms_per_launch": ms, "bytes_per_launch": alg,
            "out": "fp64" if es == 8 else "fp32", "network": "256 species x 256 reactions",
            "jacobian_nnz": int(nnz.value), "instances": n_inst,
            "write_only_ceiling_gbs": fill_gbs,
            "frac_of_write_ceiling": alg / (ms * 1e-3) / 1e9 / fill_gbs}


def run_kernels(args):
    """Single-evaluation kernels alone (RHS and Newton matrix on device
    buffers), with their HBM fractions; one JSON line.  Each kernel runs
    --warmup untimed launches, then --steps timed ones."""
    import torch
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    peaks, peak_kind = load_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    out = {"workload": "kernels", "peak_hbm_gbs": hbm, "peak_source": peak_kind}
    reps, warm = max(1, args.steps), max(1, args.warmup)
    out["rhs_hbm"] = rhs_bandwidth(torch, stream, reps=reps, warm=warm)
    for prec, key in ((0, "newton_hbm_fp64"), (1, "newton_hbm_fp32")):
        out[key] = newton_bandwidth(torch, stream, prec, reps=reps, warm=warm)
    for key in ("rhs_hbm", "newton_hbm_fp64", "newton_hbm_fp32"):
        out[key]["frac"] = out[key]["gbs"] / hbm
    print(json.dumps(out), flush=True)
    return 0


def bdf_measure(torch, stream, models, max_steps, engine):
    """The BDF controller (rtol 1e-6, atol 1e-9, orders 1-5) on the same batch
    as the headline: one persistent launch, device-resident inputs, CUDA
    events.  A different algorithm from LASSIE's loop (error control instead
    of fixed backward-Euler steps), reported beside it.  engine "fp64": FP64
    LU, bit-exact vs its CPU restatement; "mixed": FP32 Gauss-Jordan inverse
    as the Newton iteration matrix, FP64 residuals."""
    from lassie_gb300 import solver
    b = solver.Batch(models, engine=engine, max_steps=max_steps, deadline_s=900,
                     bdf={"rtol": 1e-6, "atol": 1e-9})
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        b.run(stream.cuda_stream)  # warm-up, creation order (largest network first)
        e1.record(stream)
    torch.cuda.synchronize()
    ms_creation = e0.elapsed_time(e1)
    b.order_by_cost()  # longest first by the warm-up's per-instance times
    with torch.cuda.stream(stream):
        e0.record(stream)
        b.run(stream.cuda_stream)
        e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    _, st = b.read()
    done = sum(1 for s in st if s["status"] == 0)
    ok = [s for s in st if s["status"] == 0]
    return {"sims_per_s": done / (ms * 1e-3), "ms": ms, "completed": done,
            "other_status": sorted({s["status"] for s in st if s["status"] != 0}),
            "mean_steps": sum(s["be_steps"] for s in ok) / max(1, len(ok)),
            "mean_factorisations": sum(s["lu_factorisations"] for s in ok) / max(1, len(ok)),
            "mean_newton_iters": sum(s["newton_iters"] for s in ok) / max(1, len(ok)),
            "controller": "BDF orders 1-5, rtol 1e-6, atol 1e-9", "engine": engine,
            "queue_order": "longest first by the warm-up run's per-instance times",
            "ms_creation_order": ms_creation}


def parity_table():
    """Max relative error (|a-b| / max(|b|, atol/rtol)) of the mixed form
    against the plain FP64 GPU form, which equals the CPU oracle bit for bit
    for N <= 512 (tests/test_gpu_parity.py), per configuration on horizons
    the FP64 form finishes in seconds, with both forms' step counts."""
    import numpy as np
    from lassie_gb300 import synth, solver
    cases = {
        "c1 (64 x 64, t in [0,10])": synth.make_c1(),
        "c2 (512 x 512 stiff, t in [0,0.004])": synth.shorten(synth.make_c2(), 0.004, 3),
        "c3 (4096 x 4096, t in [0,0.02])": synth.shorten(synth.make_c3(), 0.02, 3),
        # t in [0, 0.8]: on [0, 1] a one-ulp change of the Newton corrections
        # already changes this network's RKF45 step sequence
        "c5 (256 x 256, t in [0,0.8])": synth.shorten(synth.make_c5(1)[0][0], 0.8, 9),
    }
    out = {}
    for name, m in cases.items():
        a, sa = solver.simulate(m, engine="mixed", deadline_s=600)
        b, sb = solver.simulate(m, engine="fp64", deadline_s=600)
        rel = np.abs(a - b) / np.maximum(np.abs(b), ATOL / RTOL)
        out[name] = {"max_rel_err": float(rel.max()),
                     "within_rtol1e-6_atol1e-9": bool(np.all(np.abs(a - b) <= ATOL + RTOL * np.abs(b))),
                     "steps_mixed": [sa["be_steps"], sa["rkf_accepts"], sa["newton_iters"]],
                     "steps_fp64": [sb["be_steps"], sb["rkf_accepts"], sb["newton_iters"]]}
    return out


def adjoint_measure(n_copies=64):
    """Differentiation workload: 64 copies of a 256 x 256 network,
    k = 10^U(-3,3), loss = sum of squares over 40 samples in (0,10] against
    trajectories of k * exp(N(0,0.3^2)).  Returns grads/s and the cost of one
    gradient relative to one forward solve (both through the public API)."""
    from lassie_gb300 import synth, solver
    from lassie_gb300.adjoint import adjoint_batch
    base, k_t = synth.make_c5(n_copies)
    tgt_models = []
    for q, m in enumerate(base):
        mt = synth.shorten(m, 10.0, 41)
        mt.t = m.t
        mt.k = k_t[q]
        tgt_models.append(mt)
    targets, _ = solver.simulate_batch(tgt_models, engine="mixed", deadline_s=600)
    solver.simulate_batch(base, engine="mixed", deadline_s=600)  # warm-up
    t0 = time.perf_counter()
    solver.simulate_batch(base, engine="mixed", deadline_s=600)
    t_fwd = time.perf_counter() - t0
    adjoint_batch(base, targets, deadline_s=600)  # warm-up
    t0 = time.perf_counter()
    loss, gk, _, _, stats = adjoint_batch(base, targets, deadline_s=600)
    t_adj = time.perf_counter() - t0
    return {"grads_per_s": n_copies / t_adj, "forward_sims_per_s": n_copies / t_fwd,
            "adjoint_over_forward": t_adj / t_fwd, "copies": n_copies,
            "mean_loss": float(sum(loss) / len(loss)),
            "be_steps_per_copy": float(sum(s["be_steps"] for s in stats) / len(stats)),
            "workload": "c5: 64 x (256 species x 256 reactions), k~10^U(-3,3), 40 samples "
                        "in (0,10], targets from k*exp(N(0,0.3^2))"}


def run_c3(args):
    """The 4096-species network (C3) on the wide engine: one instance over
    the whole GPU, Gauss-Jordan inverse in FP32 + FP64 refinement."""
    import torch
    from lassie_gb300 import synth, solver
    from lassie_gb300 import _native as nat
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if rank != 0:
        return 0  # a single model does not shard: replicas only
    horizon = 50.0 if args.horizon == 20.0 else args.horizon
    m = synth.make_c3()
    if horizon != 50.0:
        m = synth.shorten(m, horizon, max(2, int(round(100 * horizon / 50)) + 1))
    stream = torch.cuda.Stream()
    # BF16 factors need more refinement sweeps than the default cap of 8
    refine_max = 32 if args.tensor_cores == "bf16" else 0
    batch = solver.Batch([m], engine="mixed", max_steps=args.max_steps * 10, deadline_s=1800,
                         tensor_cores=args.tensor_cores, refine_max=refine_max)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            batch.run(stream.cuda_stream)
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        with ClockSampler(local) as clocks:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for e0, e1 in evs:
                flush.zero_()
                e0.record(stream)
                batch.run(stream.cuda_stream)
                e1.record(stream)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
    kernel_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    outs, stats = batch.read()
    st = stats[0]
    wall = t1 - t0
    s0 = time.perf_counter()
    _, st_e2e = solver.simulate(m, engine="mixed", max_steps=args.max_steps * 10, deadline_s=1800,
                                tensor_cores=args.tensor_cores, refine_max=refine_max)
    e2e = 1.0 / (time.perf_counter() - s0)
    peaks, peak_kind = load_peaks()
    n = float(m.n_species)
    flops = st["lu_factorisations"] * (2.0 / 3.0) * n ** 3 + st["refine_sweeps"] * 2.0 * n * n
    k_ms = statistics.mean(kernel_ms)
    achieved = flops / (k_ms * 1e-3) / 1e12
    peak = float(peaks.get("bf16_tflops_sustained", 1700.0))
    h2d, d2h = batch.transfer_bytes()
    line = {"metric": METRIC, "value": args.steps / wall, "unit": "sims/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * wall / args.steps,
            "higher_is_better": True, "scaling": "replicas only", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded, numpy default_rng(3000))",
            "config": {"workload": f"c3: 4096 species x 4096 reactions, 2 reactants + 2 products, "
                                   f"k~10^U(-4,2), t in [0,{horizon:g}]",
                       "form": "mixed (FP32 Gauss-Jordan inverse + FP64 refinement), wide engine",
                       "tensor_cores": args.tensor_cores,
                       "l2": "flushed between steps (256 MB write)"},
            "status": st["status"],
            "steps_taken": {"be": st["be_steps"], "rkf": st["rkf_accepts"],
                            "newton": st["newton_iters"], "factorisations": st["lu_factorisations"],
                            "sweeps": st["refine_sweeps"]},
            "e2e": {"value": e2e, "unit": "sims/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": batch.launches() * args.steps,
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": None, "kernel": "wide_kernel<float>",
                         "kernel_ms": k_ms, "algorithmic_flops_per_launch": flops,
                         "peak_kind": f"{peak_kind} bf16 sustained"},
            "clocks": clocks.summary()}
    if not args.no_extras:
        line["cpu_lsoda"] = lsoda_c3()
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--instances", type=int, default=2048)
    ap.add_argument("--horizon", type=float, default=20.0,
                    help="integrate t in [0, horizon] (20 = the workload; smaller values "
                         "make small profiling cases)")
    ap.add_argument("--max-steps", type=int, default=25000,
                    help="loop-iteration cap per instance (the same for every arm)")
    ap.add_argument("--workload", default="c4", choices=["c4", "c3", "kernels"],
                    help="c4: the 2048-instance batch (default); c3: the 4096-species "
                         "network on the wide engine (t in [0, 50], or --horizon); "
                         "kernels: the RHS and Newton-matrix kernels alone")
    ap.add_argument("--tensor-cores", nargs="?", const="tf32", default="tf32",
                    choices=["off", "tf32", "bf16"],
                    help="c3: rank-32 updates of the factorisation on the FP32 pipes (off) or "
                         "on the tensor cores, with split TF32 operands (tf32, the default) or "
                         "BF16 operands and FP32 accumulation (bf16)")
    ap.add_argument("--scaling", default="weak", choices=["weak", "strong"],
                    help="weak: every rank integrates its own --instances instances "
                         "(default); strong: the ranks split one batch of --instances")
    ap.add_argument("--cpu-full-horizon", action="store_true",
                    help="run the CPU sample over the whole horizon next to its "
                         "extrapolated short-horizon figure, then exit (no GPU)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the FP64-form, RHS and CPU-baseline measurements")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.cpu_full_horizon:
        return run_cpu_full_horizon(args)
    if args.workload == "c3":
        return run_c3(args)
    if args.workload == "kernels":
        return run_kernels(args)

    import numpy as np
    import torch
    from lassie_gb300 import synth, solver, sharding
    from lassie_gb300 import _native as nat

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    L = nat.load()
    if not L.lassie_device_ok():
        raise RuntimeError("no sm_103 device")

    if args.scaling == "weak":
        # weak scaling: every rank integrates its own 2048 instances
        ids = list(sharding.weak_shard(args.instances, rank))
    else:
        # strong scaling: one fixed batch split over the ranks by cost
        ids = sharding.cost_shard(synth.c4_sizes(args.instances), world)[rank]
    models = [synth.make_c4_instance(q) for q in ids]
    if args.horizon != 20.0:
        models = [synth.shorten(m, args.horizon, max(2, int(round(50 * args.horizon / 20))))
                  for m in models]
    stream = torch.cuda.Stream()
    batch = solver.Batch(models, engine="mixed", max_steps=args.max_steps, deadline_s=900)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > L2

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    with torch.cuda.stream(stream):
        w0, w1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for w in range(args.warmup):
            flush.zero_()
            if w == args.warmup - 1:
                w0.record(stream)
            batch.run(stream.cuda_stream)
            if w == args.warmup - 1:
                w1.record(stream)
        torch.cuda.synchronize()
        ms_creation_order = w0.elapsed_time(w1) if args.warmup > 0 else None
        # the timed runs take the instances longest first, by the last
        # warm-up run's per-instance times (no result changes)
        batch.order_by_cost()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        with ClockSampler(local) as clocks:
            barrier()
            t0 = time.perf_counter()
            for e0, e1 in evs:
                flush.zero_()
                e0.record(stream)
                batch.run(stream.cuda_stream)
                e1.record(stream)
            barrier()
            t1 = time.perf_counter()
    kernel_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    outs, stats = batch.read()
    done = sum(1 for s in stats if s["status"] == 0)
    capped = sum(1 for s in stats if s["status"] == nat.ERR_MAX_STEPS)
    bad = [s["status"] for s in stats if s["status"] not in (0, nat.ERR_MAX_STEPS)]
    wall = sharding.max_over_ranks(t1 - t0)
    done_all = sharding.sum_over_ranks(done)
    value = done_all * args.steps / wall
    ms_per_step = 1000.0 * wall / args.steps

    # end to end through the public host-buffer API
    h2d, d2h = batch.transfer_bytes()
    e2e_t = []
    for _ in range(1):
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        solver.simulate_batch(models, engine="mixed", max_steps=args.max_steps, deadline_s=900)
        e2e_t.append(time.perf_counter() - s0)
    e2e_val = done / statistics.mean(e2e_t)

    # roofline of the integrator kernel (FP32 LU + FP64 refinement)
    peaks, peak_kind = load_peaks()
    flops = lu_flops(stats, models, "mixed")
    k_ms = statistics.mean(kernel_ms)
    achieved = flops / (k_ms * 1e-3) / 1e12
    peak = float(peaks.get("bf16_tflops_sustained", 1700.0))
    # the pipes that bound it: FP32 FMA (152 SMs x 128 lanes x 2 FLOP x the
    # maximum SM clock) and FP64 (the GB300's FP64 rate, 1.25 TFLOP/s nominal)
    f32, f64 = pipe_work(stats, models)
    sm_ghz = float(peaks.get("sm_max_mhz", 2070.0)) / 1000.0
    fp32_peak = 152 * 128 * 2 * sm_ghz / 1000.0
    roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": load_traffic(flops),
                "kernel": "compat_kernel<float>", "kernel_ms": k_ms,
                "algorithmic_flops_per_launch": flops,
                "peak_kind": f"{peak_kind} bf16 sustained",
                "pipes": {
                    "fp32_fma": {"achieved_tflops": f32 / (k_ms * 1e-3) / 1e12,
                                 "peak_tflops": fp32_peak,
                                 "frac": f32 / (k_ms * 1e-3) / 1e12 / fp32_peak,
                                 "flops_per_launch": f32,
                                 "peak_kind": "nominal: 152 SMs x 128 FP32 lanes x 2 x max clock"},
                    "fp64": {"achieved_tflops": f64 / (k_ms * 1e-3) / 1e12,
                             "peak_tflops": 1.25,
                             "frac": f64 / (k_ms * 1e-3) / 1e12 / 1.25,
                             "flops_per_launch": f64, "peak_kind": "nominal GB300 FP64"},
                    "note": "latency-bound: one 512-thread CTA per instance; issue and "
                            "pipe activity in the ncu summaries under profiles/"}}

    line = {"metric": METRIC, "value": value, "unit": "sims/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": args.scaling, "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded, numpy default_rng(1000*4 + instance))",
            "config": workload_config(args),
            "run": {"instances_per_gpu": len(models), "completed_instances": done_all,
                    "capped_instances": capped, "form": "mixed (FP32 LU + FP64 refinement)",
                    "tile_rows": {str(r): batch.tile_rows().count(r) for r in (8, 4, 2)},
                    "parallelism": f"instances sharded over {world} GPU(s) "
                                   f"({args.scaling} scaling)"},
            "queue_order": {"timed_steps": "longest first by the last warm-up run's per-instance "
                                           "integration times (lassie_batch_order_by_cost)",
                            "warmup_order": "largest network first (creation order)",
                            "ms_last_warmup_step": ms_creation_order},
            "failed_instances": len(bad),
            "e2e": {"value": e2e_val, "unit": "sims/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": batch.launches() * args.steps,
            "roofline": roofline,
            "clocks": clocks.summary()}

    if rank == 0 and world == 1 and not args.no_extras:
        # plain FP64 GPU form vs the mixed form on the same sample
        # (sqrt(sqrt()) quarter root, as the oracle, so that the oracle's
        # spread stored for this sample applies)
        sample = [synth.shorten(m, 2.0, 5) for m in models[::13][:152]]
        res = {}
        for eng in ("fp64", "mixed"):
            b = solver.Batch(sample, engine=eng, max_steps=args.max_steps // 10, deadline_s=900,
                             root="sqrt")
            b.run(stream.cuda_stream)
            b.sync()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                flush.zero_()
                e0.record(stream)
                b.run(stream.cuda_stream)
                e1.record(stream)
            torch.cuda.synchronize()
            o, st = b.read()
            res[eng] = (e0.elapsed_time(e1), o, st)
        worst, nbad = max_rel_err(res["mixed"][1], res["fp64"][1])
        # instances whose two forms took the same step sequence, and the rest
        # (a rounding-driven step decision went the other way)
        key = lambda st: (st["be_steps"], st["rkf_accepts"], st["newton_iters"])  # noqa: E731
        same = [q for q, (a, b) in enumerate(zip(res["mixed"][2], res["fp64"][2]))
                if key(a) == key(b)]
        w_same, n_same = max_rel_err([res["mixed"][1][q] for q in same],
                                     [res["fp64"][1][q] for q in same])
        line["fp64_form"] = {
            "sample": f"{len(sample)} instances (every 13th), t in [0,2] (0.1 of horizon)",
            "fp64_ms": res["fp64"][0], "mixed_ms": res["mixed"][0],
            "speedup_mixed_vs_fp64": res["fp64"][0] / res["mixed"][0],
            "max_rel_err_vs_fp64": worst, "points_outside_rtol1e-6_atol1e-9": nbad,
            "instances_same_step_sequence": len(same),
            "max_rel_err_same_step_sequence": w_same,
            "points_outside_same_step_sequence": n_same,
            "oracle_spread": spread_classes(res["mixed"][1], res["fp64"][1], res["mixed"][2],
                                            args.max_steps // 10)}
        line["parity_vs_fp64_form"] = parity_table()
        line["adjoint"] = adjoint_measure()
        line["rhs_hbm"] = rhs_bandwidth(torch, stream)
        line["rhs_hbm"]["frac"] = line["rhs_hbm"]["gbs"] / float(peaks.get("hbm_gbs", 6800.0))
        for prec, key in ((0, "newton_hbm_fp64"), (1, "newton_hbm_fp32")):
            line[key] = newton_bandwidth(torch, stream, prec)
            line[key]["frac"] = line[key]["gbs"] / float(peaks.get("hbm_gbs", 6800.0))
        line["bdf_controller"] = {eng: bdf_measure(torch, stream, models, args.max_steps, eng)
                                  for eng in ("mixed", "fp64")}
        line["cpu_lsoda"] = lsoda_baseline(args.instances, stride=64)
        line["cpu_baseline"] = cpu_baseline(args.instances, max_steps=args.max_steps)
        line["cpu_baseline"].pop("seconds", None)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
