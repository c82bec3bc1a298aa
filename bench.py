#!/usr/bin/env python3
"""Benchmark of the coupled thermal MRT-LBM time step on GB300.

Workload: 3D Rayleigh-Benard cube, D3Q19 MRT flow + D3Q7 MRT temperature, 256^3 cells,
no-slip walls, adiabatic side walls, hot bottom (+0.5) / cold top (-0.5), Ra = 1e7,
Pr = 0.71, free-fall velocity U = 0.1, linear T + seeded 1e-3 noise.  A "step" is one
coupled (flow + thermal) time step over the whole lattice; MLUPS counts one coupled cell
update as one, as the reference's runtime print does (3DRB.F90:303-305).

Headline `value`: the plain method to FP64 accuracy, through the fused kernels of the fixed
arithmetic (q60 integers on the integer pipes; within 1e-12 of the reference's populations
after 1000 steps, within 1e-10 in Nu), inputs resident in HBM.  Beside it: the plain method
in the reference's own FP64 operations (bit for bit the reference), and the FP32 / FP16
storage forms.  `e2e` is the headline metric through the C ABI with host buffers in the
reference's Fortran layout (state in, steps, T field and Nu/Re out).  `cpu_baseline` is the
C++ restatement of the reference's OpenMP CPU path timed on this host's cores; the GPU then
runs the same steps with the reference's arithmetic and the two temperature fields are
compared bit for bit.  The 128^3 cube is a secondary leg (`cube128`).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.join(ROOT, "-2d-3d-_gb300")
for _p in (ROOT, PKG_ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "coupled MLUPS (D3Q19/D3Q7 MRT-LBM step)"
UNIT = "MLUPS"
N_CELL_EDGE = 256
BYTES_PER_CELL = {"fp64": 416, "fp64x": 416, "fp32": 208, "fp16": 104}  # populations read + written once
# FP64 work of the plain method per coupled cell update (3D), counted by ncu on the fused
# kernels (sass thread instructions, flow + thermal): dadd 398, dmul 103, dfma 57.  Products
# with exact powers of two run on the integer pipes and are not counted.
FP64_INST_PER_CELL = 398 + 103 + 57
FP64_FLOP_PER_CELL = 398 + 103 + 2 * 57
DTYPE = {"fp64": "f64", "fp64x": "i64 fixed-point 2^-60 (FP64 accuracy)", "fp32": "f32",
         "fp16": "f16-storage/f32-arith"}
FALLBACK_HBM_GBS = 6800.0


def workload_params(precision="fp64", n=N_CELL_EDGE):
    from lbmgpu.abi import rb_params
    return rb_params(dim=3, n=n, Ra=1e7, Pr=0.71, U=0.1, noise_amp=1e-3, seed=20261203, precision=precision)


# Kernels one steady-state step launches (inside the replayed graphs as well): the fixed
# arithmetic's interior-row and face-row kernels for the flow and the thermal half; the
# plain method's flow and thermal kernels; the FP32/FP16 flow and thermal kernels and the
# step counter of the stochastic rounding.
LAUNCHES_PER_STEP = {"fp64x": 4, "fp64": 2, "fp32": 3, "fp16": 3}


def workload_config(n=N_CELL_EDGE):
    return {
        "workload": "3D Rayleigh-Benard cube D3Q19/D3Q7 MRT, %d^3 cells, Ra=1e7, Pr=0.71, U=0.1, no-slip walls, "
                    "adiabatic sides, T linear + 1e-3 seeded noise (seed 20261203)" % n,
        "cells": n ** 3,
        "l2": "inputs larger than L2 (populations per step: FP64 %.0f MB, FP32 %.0f MB, FP16 %.0f MB; L2 129 MB)"
              % (416 * n ** 3 / 1e6, 208 * n ** 3 / 1e6, 104 * n ** 3 / 1e6),
        "step": "one coupled flow+thermal time step over the whole lattice",
    }


def measured_hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(cells):
    """DRAM bytes per step (flow + thermal launch) of each storage form from the committed ncu
    capture, scaled to `cells` by the cells it was captured on; None when absent."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(path) as fh:
            data = json.load(fh)
    except Exception:
        return {}
    return {prec: v["bytes_per_step"] * cells / v["cells"] for prec, v in data.items() if isinstance(v, dict)}


def fp64_peak_tflops():
    """cuBLAS DGEMM (8192^3, best of 3) on this GPU: the FP64 denominator of the plain method."""
    import torch
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    c = a @ b
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = float("inf")
    for _ in range(3):
        e0.record()
        c = a @ b
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b, c
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(steps=None, budget_s=12.0, n=N_CELL_EDGE, device=None):
    """C++ restatement of the reference's 8-pass OpenMP CPU step, all host cores, bounded sample.
    With a device: the GPU plain method then runs the same steps from the same initial state
    and the final temperature fields are compared bit for bit."""
    from oracle import oracle as ora
    threads = ora.set_threads(os.cpu_count() or 1)
    p = workload_params("fp64", n)
    o = ora.Oracle(p)
    o.initial()
    o.step(1)
    t0 = time.perf_counter()
    done = 0
    if steps is not None:
        o.step(steps)
        done = steps
    else:
        while time.perf_counter() - t0 < budget_s:
            o.step(2)
            done += 2
    dt = time.perf_counter() - t0
    cells = n ** 3
    out = {"value": cells * done / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": "%d steps of the %d^3 workload (%.1f s), C++ restatement of the reference's OpenMP "
                     "8-pass step (-O3 -fopenmp), %d threads" % (done, n, dt, threads)}
    if device is not None:
        import numpy as np
        import lbmgpu
        from lbmgpu.abi import FIELDS, field_shape
        lat = lbmgpu.Lattice(p, device=device)
        lat.initial()
        lat.step(1 + done)
        t_gpu = lat.get_state("T")
        lat.close()
        out["gpu_check"] = {"steps": 1 + done,
                            "T_bitwise_equal": bool(np.array_equal(t_gpu, o.get(FIELDS["T"], field_shape(p, "T"))))}
    o.close()
    return out


def run_reference(args):
    rank, world, local, pg = dist_setup(args)
    if rank != 0:
        return 0
    from oracle import oracle as ora
    ora.build()
    threads = ora.set_threads(os.cpu_count() or 1)
    o = ora.Oracle(workload_params("fp64", args.size))
    o.initial()
    o.step(args.warmup)
    t0 = time.perf_counter()
    o.step(args.steps)
    dt = time.perf_counter() - t0
    cells = args.size ** 3
    value = cells * args.steps / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload_config(args.size),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d steps of the %d^3 workload after %d warm-up steps; C++ restatement of the "
                                   "reference's OpenMP CPU path (the Fortran cannot be compiled here)"
                                   % (args.steps, args.size, args.warmup)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def time_precision(prec, args, pg, local, size=None):
    import torch
    import lbmgpu
    p = workload_params(prec, size or args.size)
    lat = lbmgpu.Lattice(p, device=local)
    lat.initial()
    lat.step(args.warmup)
    lat.sync()
    stream = torch.cuda.ExternalStream(lat.stream_handle(), device=torch.device("cuda", local))
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(pg)
    torch.cuda.synchronize()
    start.record(stream)
    lat.step(args.steps)
    end.record(stream)
    end.synchronize()
    torch.cuda.synchronize()
    barrier(pg)
    ms = start.elapsed_time(end)
    ms = max_over_ranks(pg, ms)
    # per-kernel device times (no graph), for the roofline of the fused step
    ms_flow, ms_thermal = lat.time_kernels(min(args.steps, 20))
    nu, re = lat.calNuRe()
    lat.close()
    cells = p.nx * p.ny * p.nz
    return {"ms_total": ms, "ms_per_step": ms / args.steps, "mlups": cells * args.steps / (ms / 1e3) / 1e6,
            "ms_flow": ms_flow, "ms_thermal": ms_thermal, "Nu": nu, "Re": re}


def e2e_run(prec, args, local, jobs=3):
    """State in from host arrays (Fortran layout), K steps, T field and Nu/Re out, via the C ABI.
    The whole job runs `jobs` times back to back (each with every transfer); the median job
    gives the value, and every job's time is listed."""
    import numpy as np
    import lbmgpu
    p = workload_params(prec, args.size)
    lat = lbmgpu.Lattice(p, device=local)
    lat.initial()
    names = ["f", "g", "rho", "u", "v", "w", "T", "Bx_prev", "By_prev", "Bz_prev"]
    host = {k: np.ascontiguousarray(lat.get_state(k)) for k in names}
    lat.step(args.warmup)
    lat.sync()
    times = []
    for _ in range(jobs):
        t0 = time.perf_counter()
        for k in names:
            lat.set_state(k, host[k])
        lat.step(args.steps)
        T = lat.get_state("T")
        nu, re = lat.calNuRe()
        times.append(time.perf_counter() - t0)
    lat.close()
    dt = sorted(times)[len(times) // 2]
    h2d = sum(a.nbytes for a in host.values())
    d2h = T.nbytes + 16
    cells = p.nx * p.ny * p.nz
    return {"value": cells * args.steps / dt / 1e6, "unit": UNIT, "h2d_bytes_per_step": h2d / args.steps,
            "d2h_bytes_per_step": d2h / args.steps,
            "job": "lbm_set_state x%d (Fortran-layout host arrays) + lbm_step(%d) + lbm_get_state(T) + lbm_calNuRe"
                   % (len(names), args.steps),
            "jobs_ms": [round(t * 1e3, 1) for t in times], "statistic": "median of %d jobs" % jobs}


def plain_rate_2d(local, ny=128):
    """FP64 plain-method MLUPS on a 2D cell (for the served-form comparison)."""
    import lbmgpu
    from lbmgpu.abi import rb_params
    lat = lbmgpu.Lattice(rb_params(dim=2, ny=ny, Ra=1e5, noise_amp=1e-3), device=local)
    lat.initial()
    lat.step(64)
    lat.sync()
    t0 = time.perf_counter()
    lat.step(3200)
    lat.sync()
    dt = time.perf_counter() - t0
    lat.close()
    return 2 * ny * ny * 3200 / dt / 1e6


def run_sampled(p, local, steps, every):
    """One lattice run alone for `steps` steps, calNuRe sampled every `every` steps; returns
    (seconds on the device stream, [(step, Nu)], diverged)."""
    import torch
    import lbmgpu
    lat = lbmgpu.Lattice(p, device=local)
    lat.initial()
    stream = torch.cuda.ExternalStream(lat.stream_handle(), device=torch.device("cuda", local))
    hist, diverged = [], False
    t_dev = 0.0
    done = 0
    while done < steps:
        k = min(every, steps - done)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        lat.step(k)
        b.record(stream)
        b.synchronize()
        t_dev += a.elapsed_time(b) / 1e3
        done += k
        try:
            hist.append((done, lat.calNuRe()[0]))
        except lbmgpu.LbmDiverged:
            diverged = True
            break
    lat.close()
    return t_dev, hist, diverged


def tail_mean(hist, from_step):
    xs = [nu for s, nu in hist if s > from_step]
    return sum(xs) / len(xs) if xs else None


def ensemble_run(args, local, steps_total=13000, every=500):
    """Batched form (the many-instance 2D workload): 64 D2Q9/D2Q5 RB instances, aspect 2, ny drawn from
    {64,...,512}, Ra log-uniform in [1e4, 1e8], Pr in {0.71, 7}, U = 0.1, FP32 storage, one
    launch per stage over a packed tile table, graph replay, autotuned tiles.  Every member's
    Nu is sampled every `every` steps; each member is then run alone at FP64 accuracy (the
    fixed arithmetic, which stays within 1e-12 of the plain method's populations) and the
    time-averaged Nu of the second half of the run is compared member by member."""
    import random
    import torch
    import lbmgpu
    from lbmgpu.abi import rb_params
    rng = random.Random(20261203)
    specs = []
    for m in range(64):
        ny = rng.choice([64, 96, 128, 192, 256, 384, 512])
        ra = math.exp(rng.uniform(math.log(1e4), math.log(1e8)))
        pr = rng.choice([0.71, 7.0])
        specs.append(dict(dim=2, ny=ny, nx=2 * ny, Ra=ra, Pr=pr, U=0.1, noise_amp=1e-3, seed=20261203 + m))
    ens = lbmgpu.Ensemble(device=local)
    lats = []
    for sp in specs:
        lat = lbmgpu.Lattice(rb_params(precision="fp32", **sp), device=local)
        lat.initial()
        ens.add(lat)
        lats.append(lat)
    cells = sum(2 * sp["ny"] * sp["ny"] for sp in specs)
    cfg = ens.autotune(3)
    ens.step(10)
    ens.sync()
    stream = torch.cuda.ExternalStream(ens.stream_handle(), device=torch.device("cuda", local))
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k = 320
    a.record(stream)
    ens.step(k)
    b.record(stream)
    b.synchronize()
    ms = a.elapsed_time(b)
    mlups = cells * k / (ms / 1e3) / 1e6
    # run every member on to steps_total, sampling Nu at multiples of `every`
    hist = {m: [] for m in range(64)}
    diverged = {}
    while lats[0].itc < steps_total:
        done = lats[0].itc
        nxt = min(steps_total, (done // every + 1) * every)
        ens.step(nxt - done)
        ens.sync()
        for m, lat in enumerate(lats):
            if m in diverged:
                continue
            try:
                hist[m].append((lat.itc, lat.calNuRe()[0]))
            except lbmgpu.LbmDiverged:
                diverged[m] = lat.itc
    ens.close()
    for lat in lats:
        lat.close()
    # the same members at FP64 accuracy (the fixed arithmetic), one stream per member
    from lbmgpu.server import StreamBatch
    xl = [lbmgpu.Lattice(rb_params(precision="fp64x", **sp), device=local) for sp in specs]
    sb = StreamBatch()
    for lat in xl:
        lat.initial()
        sb.add(lat)
    sb.step(64)
    sb.sync()
    t0 = time.perf_counter()
    sb.step(k)
    sb.sync()
    fp64x_mlups = cells * k / (time.perf_counter() - t0) / 1e6
    for lat in xl:
        lat.close()
    half = steps_total // 2
    members = []
    for m, sp in enumerate(specs):
        rec = {"member": m, "ny": sp["ny"], "Ra": sp["Ra"], "Pr": sp["Pr"]}
        if m in diverged:
            rec["diverged_fp32_at"] = diverged[m]
            members.append(rec)
            continue
        _, h64, div64 = run_sampled(rb_params(precision="fp64x", **sp), local, steps_total, every)
        rec["Nu_fp32_batched"] = tail_mean(hist[m], half)
        rec["Nu_fp64"] = tail_mean(h64, half) if not div64 else None
        if rec["Nu_fp64"] is not None and rec["Nu_fp32_batched"] is not None:
            rec["rel_dNu"] = abs(rec["Nu_fp32_batched"] - rec["Nu_fp64"]) / abs(rec["Nu_fp64"])
        members.append(rec)
    good = [r["rel_dNu"] for r in members if "rel_dNu" in r and r["Nu_fp64"] >= 1.0]
    unphys = [r["member"] for r in members if r.get("Nu_fp64") is not None and r["Nu_fp64"] < 1.0]
    good.sort()
    return {"workload": "64 D2Q9/D2Q5 RB instances, aspect 2, ny in {64..512}, Ra log-uniform 1e4..1e8, "
                        "Pr in {0.71,7}, FP32 storage, %d cells" % cells,
            "aggregate_mlups": mlups, "ms_per_step": ms / k, "steps_timed": k, "autotuned": cfg,
            "fp64_accuracy_streams_mlups": fp64x_mlups,
            "fp64_accuracy_note": "the same members at FP64 accuracy (fixed arithmetic), one lbm_step per member "
                                  "on its own stream, %d steps, wall clock" % k,
            "launches_per_step": 3,  # flow, thermal, step counters (one member list: all 2D, even nx)
            "dNu_vs_fp64": {
                "compared": len(good), "median": good[len(good) // 2] if good else None,
                "max": good[-1] if good else None, "within_1pct": sum(1 for x in good if x <= 0.01),
                "excluded_unphysical_fp64_Nu_below_1": unphys,
                "how": "time-averaged Nu over steps %d..%d sampled every %d steps; FP64 reference: each member "
                       "alone with the fixed arithmetic (FP64 accuracy)" % (half, steps_total, every)},
            "members": members,
            "diverged": {"count": len(diverged), "note": "under-resolved draws (tau_f close to 1/2) reported as "
                                                         "LBM_ERR_DIVERGED"}}


def served_run(args, local, precision="fp32"):
    """Served form (the Poisson solve stream): Poisson arrivals at 2/s, half 2D (ny 64..512, aspect 2)
    half 3D (n 64..192), Ra log-uniform 1e4..1e8, Pr in {0.71, 7}, admission by an 80% HBM
    budget, each solve run until its windowed-mean Nu changes by < 0.1% between consecutive
    windows, or a step cap.  FP32 storage runs as the batched form; FP64 accuracy ("fp64x",
    the fixed arithmetic) runs each solve with its own lbm_step on its own stream.  The default
    run is scaled to fit a bench (20 s of arrivals, 1000-step window, 4000-step cap);
    --served-full runs the configuration as stated (600 s, 5000-step window).  A seeded random
    sample of the served requests is then run one at a time with the plain FP64 method and
    with the fixed arithmetic for the same steps: their measured solves/h, and |dNu| of the
    windowed means (FP32 streams against the fixed arithmetic, the FP64-accuracy stream
    against the plain method)."""
    import random
    import lbmgpu
    from lbmgpu import server as srv
    duration, drain = args.served_seconds, args.served_drain
    window, cap = args.served_window, args.served_cap
    chunk = 500
    reqs = srv.poisson_requests(2.0, duration)
    for q in reqs:
        q.precision = precision
    s = srv.SolveServer(device=local, chunk_steps=chunk, window=window, rel_tol=1e-3, max_steps=cap,
                        autotune=False, precision=precision)
    t0 = time.perf_counter()
    results = s.run(reqs, time_limit=duration + drain)
    wall = time.perf_counter() - t0
    finished = {r.rid for r in results}
    unfinished = len(reqs) - len(finished)
    summary = srv.summarize(results, wall, s.cell_steps)
    peak = (s.peak_active, s.peak_queue)
    s.close()
    by_id = {r.rid: r for r in reqs}
    ran = [r for r in results if r.steps > 0 and not r.diverged]
    # the sample: converged solves first (their windowed mean is steady, so FP32 against FP64
    # compares like with like), then capped ones, which stopped inside a transient
    rng = random.Random(7)
    conv = [r for r in ran if r.converged]
    capd = [r for r in ran if not r.converged]
    sample = rng.sample(conv, min(len(conv), args.served_sample))
    sample += rng.sample(capd, min(len(capd), args.served_sample - len(sample)))
    plain = {"fp64": [0.0, 0], "fp64x": [0.0, 0]}
    dnu = []
    t_budget = time.perf_counter() + args.served_plain_budget
    for r in sample:
        if time.perf_counter() > t_budget:
            break
        q = by_id[r.rid]
        rec = {"rid": r.rid, "dim": q.dim, "n": q.n, "Ra": q.Ra, "Pr": q.Pr, "steps": r.steps,
               "converged": r.converged}
        last = [nu for st, nu in r.nu_history if st > r.steps - window]
        rec["Nu_served"] = sum(last) / len(last) if last else None
        for prec in ("fp64x", "fp64"):
            t, h, div = run_sampled(q.params(prec), local, r.steps, chunk)
            plain[prec][0] += t
            plain[prec][1] += 1
            rec["s_" + prec] = t
            # the reference of the comparison: FP64 accuracy for reduced-precision streams,
            # the plain FP64 method for the FP64-accuracy stream
            if prec == ("fp64" if precision == "fp64x" else "fp64x") and not div:
                rec["Nu_fp64"] = tail_mean(h, r.steps - window)
        if rec.get("Nu_fp64") and rec["Nu_served"] is not None:
            rec["rel_dNu"] = abs(rec["Nu_served"] - rec["Nu_fp64"]) / abs(rec["Nu_fp64"])
        dnu.append(rec)
    rel = sorted(x["rel_dNu"] for x in dnu if "rel_dNu" in x and x["converged"])
    rel_cap = sorted(x["rel_dNu"] for x in dnu if "rel_dNu" in x and not x["converged"])
    summary.update({
        "workload": "Poisson arrivals 2/s for %.0f s, 50/50 2D (ny 64..512, aspect 2) / 3D (n 64..192), Ra "
                    "log-uniform 1e4..1e8, Pr {0.71,7}, %s, 80%% HBM budget, stop when the %d-step windowed mean "
                    "of Nu changes < 0.1%% or at %d steps; drain limit %.0f s%s" % (
                        duration, {"fp32": "FP32 (batched)", "fp16": "FP16 (batched)",
                                   "fp64x": "FP64 accuracy (fixed arithmetic, one stream per solve)"}.get(
                            precision, precision), window, cap, drain,
                        "" if args.served_full else " (scaled from 600 s / 5000-step window)"),
        "arrived": len(reqs), "unfinished_at_limit": unfinished, "wall_s": wall,
        "peak_active": peak[0], "peak_queue": peak[1],
        "one_at_a_time_sample": {
            "requests": len(dnu), "of": len(ran),
            "plain_fp64_solves_per_hour": 3600.0 * plain["fp64"][1] / plain["fp64"][0] if plain["fp64"][0] else None,
            "fixed_fp64_solves_per_hour": 3600.0 * plain["fp64x"][1] / plain["fp64x"][0] if plain["fp64x"][0]
            else None,
            "note": "each sampled request run alone for the steps it ran served, device time only (no queueing); "
                    "served solves/h are whole-run wall-clock rates of a different mix, so compare rates per "
                    "solve of the same sample via served_vs_plain below"},
        "dNu_vs_fp64": {"converged_compared": len(rel), "median": rel[len(rel) // 2] if rel else None,
                        "max": rel[-1] if rel else None, "within_1pct": sum(1 for x in rel if x <= 0.01),
                        "capped_compared": len(rel_cap),
                        "capped_median": rel_cap[len(rel_cap) // 2] if rel_cap else None,
                        "solves": dnu,
                        "how": ("windowed mean of Nu over the solve's last window: served %s vs the same request "
                                "alone %s for the same steps; capped solves stopped inside a transient and are "
                                "listed apart" % (precision, "with the plain FP64 method" if precision == "fp64x"
                                                  else "at FP64 accuracy (fixed arithmetic)"))},
    })
    # throughput of the same sampled work: served aggregate cell updates/s against one at a time
    if plain["fp64"][0] and dnu:
        work = sum(by_id[x["rid"]].cells * x["steps"] for x in dnu)
        summary["served_vs_plain"] = {
            "served_aggregate_mlups": summary["aggregate_mlups"],
            "plain_fp64_mlups_one_at_a_time": work / plain["fp64"][0] / 1e6,
            "fixed_fp64_mlups_one_at_a_time": work / plain["fp64x"][0] / 1e6 if plain["fp64x"][0] else None}
    return summary


def at_size_run(args, local, peak, n=384, steps=40):
    """The 384^3 configuration (Ra 1e9, U 0.07): FP16 / FP32 / FP64 storage in the in-place
    (AA) pattern beside the two-buffer pattern -- throughput, device footprint, per-sweep
    kernel times, and the AA state after the same steps against FP64 AA (a short run: the
    time-averaged Nu of 200,000 steps is not a bench leg)."""
    import numpy as np
    import torch
    import lbmgpu
    from lbmgpu.abi import rb_params
    out = {"workload": "3D Rayleigh-Benard cube D3Q19/D3Q7 MRT, %d^3 cells, Ra=1e9, Pr=0.71, U=0.07, no-slip walls, "
                       "adiabatic sides, T linear + 1e-3 seeded noise" % n, "cells": n ** 3,
           "steps_each": steps + 6}
    traffic = ncu_traffic(n ** 3)
    T = {}
    for prec in ("fp16", "fp32", "fp64"):
        out[prec] = {}
        for pat in ("AB", "AA"):
            p = rb_params(dim=3, n=n, Ra=1e9, Pr=0.71, U=0.07, noise_amp=1e-3, seed=20261203, precision=prec,
                          pattern=pat)
            lat = lbmgpu.Lattice(p, device=local)
            lat.initial()
            lat.step(4)
            lat.sync()
            stream = torch.cuda.ExternalStream(lat.stream_handle(), device=torch.device("cuda", local))
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            t0.record(stream)
            lat.step(steps)
            t1.record(stream)
            t1.synchronize()
            ms = t0.elapsed_time(t1)
            tf, tt = lat.time_kernels(2)  # one even and one odd step
            nu, re = lat.calNuRe()
            rate = n ** 3 * steps / (ms / 1e3)  # cell updates / s, graph-replayed steps
            key = prec if pat == "AB" else prec + "_aa"
            achieved = BYTES_PER_CELL[prec] * rate / 1e9
            out[prec][pat] = {"mlups": rate / 1e6, "ms_per_step": ms / steps,
                              "ms_flow_thermal_mean_of_2": [tf, tt], "footprint_GB": lbmgpu.footprint(p) / 1e9,
                              "Nu": nu, "Re": re,
                              "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                           "frac": achieved / peak, "traffic": traffic.get(key),
                                           "algorithmic_bytes_per_cell": BYTES_PER_CELL[prec]}}
            if pat == "AA":
                T[prec] = (lat.get_state("T"), nu, re)
            lat.close()
    t64, nu64, re64 = T["fp64"]
    dev = np.linalg.norm(t64 - np.mean(t64))
    for prec in ("fp16", "fp32"):
        t, nu, re = T[prec]
        out[prec]["vs_fp64_AA"] = {"T_L2_rel": float(np.linalg.norm(t - t64) / dev),
                                   "dNu_rel": abs(nu - nu64) / abs(nu64), "dRe_rel": abs(re - re64) / abs(re64)}
    return out


def mean_and_se(xs, batches=10):
    """Mean of a time series and its standard error from batch means (consecutive blocks),
    which accounts for the correlation of neighbouring samples of a chaotic flow."""
    import numpy as np
    x = np.asarray(xs, dtype=np.float64)
    if x.size == 0:
        return None, None
    nb = min(batches, x.size)
    blocks = np.array_split(x, nb)
    means = np.array([b.mean() for b in blocks])
    se = float(means.std(ddof=1) / math.sqrt(nb)) if nb > 1 else None
    return float(x.mean()), se


def time_series_run(p, local, steps, every, tail_frac):
    """Advance one lattice `steps` steps, sampling the calNuRe volume Nu and Re every `every`
    steps (as the reference appends NuVolAvg(t) on every call, 3DRB.F90:1753-1770); returns
    the series and the mean and standard error over the last `tail_frac` of the samples."""
    import lbmgpu
    lat = lbmgpu.Lattice(p, device=local)
    lat.initial()
    series = []
    t0 = time.perf_counter()
    diverged = None
    for s in range(every, steps + 1, every):
        lat.step(every)
        try:
            nu, re = lat.calNuRe()
        except lbmgpu.LbmDiverged as e:
            diverged = {"step": s, "error": str(e)}
            break
        series.append((s, nu, re))
    lat.sync()
    wall = time.perf_counter() - t0
    lat.close()
    tail = series[int(len(series) * (1.0 - tail_frac)):]
    nu_m, nu_se = mean_and_se([x[1] for x in tail])
    re_m, re_se = mean_and_se([x[2] for x in tail])
    return {"steps": series[-1][0] if series else 0, "wall_s": wall, "samples_averaged": len(tail),
            "Nu_mean": nu_m, "Nu_se": nu_se, "Re_mean": re_m, "Re_se": re_se, "diverged": diverged,
            "series": series}


def accuracy_run(args, local):
    """Time-averaged Nu and Re of the storage forms against FP64 on one configuration.

    cube128: the 128^3 cube at Ra 1e7 (U 0.1); cube384: the 384^3 cube at Ra 1e9 (U 0.07,
    in-place pattern).  Each run samples calNuRe every `every` steps and averages the last
    `tail` fraction; the standard error comes from batch means.  Two seeds per storage form
    give the spread of the time average that the chaotic flow itself produces, against which
    |dNu| between storage forms is read."""
    from lbmgpu.abi import rb_params
    cfg = args.accuracy
    if cfg == "cube128":
        base = dict(dim=3, n=128, Ra=1e7, Pr=0.71, U=0.1, noise_amp=1e-3, pattern="AB")
        default_steps, tail = 150000, 0.5
    else:
        base = dict(dim=3, n=384, Ra=1e9, Pr=0.71, U=0.07, noise_amp=1e-3, pattern="AA")
        default_steps, tail = 200000, 0.2
    steps = args.accuracy_steps or default_steps
    every = args.accuracy_every
    runs = {}
    for item in args.accuracy_forms.split(","):
        prec, _, seed_tag = item.partition(":")
        seed = 20261203 + (int(seed_tag) if seed_tag else 0)
        p = rb_params(precision=prec, seed=seed, **base)
        if prec == "fp64x":
            p.pattern = 0  # the fixed arithmetic runs the two-buffer pattern
        key = "%s:seed%d" % (prec, seed)
        runs[key] = time_series_run(p, local, steps, every, tail)
        runs[key]["precision"] = prec
        runs[key]["seed"] = seed
        print(json.dumps({"accuracy_run": key, "Nu_mean": runs[key]["Nu_mean"], "Nu_se": runs[key]["Nu_se"],
                          "Re_mean": runs[key]["Re_mean"], "wall_s": runs[key]["wall_s"]}), file=sys.stderr,
              flush=True)
    ref_key = next((k for k in runs if runs[k]["precision"] == args.accuracy_ref), None)
    cmp = {}
    if ref_key is not None and runs[ref_key]["Nu_mean"]:
        r = runs[ref_key]
        for k, x in runs.items():
            if k == ref_key or x["Nu_mean"] is None:
                continue
            cmp[k] = {
                "dNu_rel": abs(x["Nu_mean"] - r["Nu_mean"]) / abs(r["Nu_mean"]),
                "dNu_rel_se": math.hypot(x["Nu_se"] or 0.0, r["Nu_se"] or 0.0) / abs(r["Nu_mean"]),
                "dRe_rel": abs(x["Re_mean"] - r["Re_mean"]) / abs(r["Re_mean"]),
                "dRe_rel_se": math.hypot(x["Re_se"] or 0.0, r["Re_se"] or 0.0) / abs(r["Re_mean"]),
            }
    out = {"accuracy": cfg, "workload": base, "steps": steps, "sample_every": every, "tail_fraction": tail,
           "reference_run": ref_key, "vs_reference": cmp,
           "runs": {k: {kk: vv for kk, vv in v.items() if kk != "series"} for k, v in runs.items()}}
    if args.accuracy_series:
        with open(args.accuracy_series, "w") as fh:
            json.dump({k: v["series"] for k, v in runs.items()}, fh)
    print(json.dumps(out))
    return 0


def rb2d_run(args, local, steps=20000, cpu_steps=20000):
    """The 2D reference case (256 x 128, x-periodic, Ra 1e5, Pr 0.71, U 0.1, plain FP64): its
    full 20,000 steps on the GPU through lbm_step, the wall-averaged Nu and volume Re at the
    end, and the same 20,000 steps of the CPU oracle (about 2.5 s on 16 host threads), with
    the final temperature field compared bit for bit and Nu, Re (reductions) to 1e-12."""
    import numpy as np
    import torch
    import lbmgpu
    from lbmgpu.abi import FIELDS, field_shape, rb_params
    from oracle import oracle as ora
    p = rb_params(dim=2, nx=256, ny=128, Ra=1e5, Pr=0.71, U=0.1, noise_amp=1e-3, seed=20261203)
    lat = lbmgpu.Lattice(p, device=local)
    lat.initial()
    lat.sync()
    stream = torch.cuda.ExternalStream(lat.stream_handle(), device=torch.device("cuda", local))
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    lat.step(steps)
    b.record(stream)
    b.synchronize()
    ms = a.elapsed_time(b)
    nu, re = lat.calNuRe()
    wall = lat.RBcalc_Nu_wall_avg()
    t_gpu = lat.get_state("T") if cpu_steps == steps else None
    lat.close()
    threads = ora.set_threads(os.cpu_count() or 1)
    o = ora.Oracle(p)
    o.initial()
    t0 = time.perf_counter()
    o.step(cpu_steps)
    dt = time.perf_counter() - t0
    cells = 256 * 128
    cpu = {"threads": threads, "steps": cpu_steps, "s": dt, "mlups": cells * cpu_steps / dt / 1e6,
           "s_for_all_steps": dt * steps / cpu_steps}
    if t_gpu is not None:
        # the fields bit for bit; Nu and Re are sums that the GPU reduces in another order
        nu_o, re_o, _ = o.calNuRe()
        cpu["T_bitwise_equal_to_gpu"] = bool(np.array_equal(t_gpu, o.get(FIELDS["T"], field_shape(p, "T"))))
        cpu["Nu_Re_rel_diff_to_gpu"] = max(abs(nu - nu_o) / abs(nu_o), abs(re - re_o) / abs(re_o))
    o.close()
    return {"workload": "2D RB D2Q9/D2Q5, 256 x 128, x periodic, Ra 1e5, Pr 0.71, U 0.1, FP64 plain method, "
                        "T linear + 1e-3 seeded noise, %d steps" % steps,
            "gpu_s": ms / 1e3, "mlups": cells * steps / (ms / 1e3) / 1e6, "Nu_volume": nu, "Re": re,
            "Nu_hot_wall": wall["Nu_hot"], "Nu_cold_wall": wall["Nu_cold"], "cpu_oracle": cpu}


def run_gpu(args):
    rank, world, local, pg = dist_setup(args)
    import torch
    torch.cuda.set_device(local)
    from lbmgpu import build as lbuild
    lbuild.build()
    peak, peak_kind = measured_hbm_peak()
    traffic = ncu_traffic(args.size ** 3)
    results = {}
    precs = [x for x in args.precisions.split(",") if x]
    with ClockSampler(local) as clk:
        for prec in precs:
            results[prec] = time_precision(prec, args, pg, local)
    clocks = clk.summary()
    e2e = None if args.no_e2e else e2e_run(precs[0], args, local)
    cells = args.size ** 3

    def roof(prec):
        r = results[prec]
        step_ms = r["ms_flow"] + r["ms_thermal"]
        achieved = BYTES_PER_CELL[prec] * cells / (step_ms / 1e3) / 1e9
        t = traffic.get(prec)
        if r["ms_thermal"] == 0.0:
            desc = "single fused kernel k_fused, %.4f ms per launch (one launch per step)" % r["ms_flow"]
        else:
            desc = "two-kernel step: flow kernel %.4f ms + thermal kernel %.4f ms per launch" % (
                r["ms_flow"], r["ms_thermal"])
        return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": t, "peak_kind": peak_kind, "kernel": desc,
                "algorithmic_bytes_per_cell": BYTES_PER_CELL[prec]}

    def roof_fp64():
        # the plain method's bound: FP64 issue (DRAM stays below 11% busy)
        r = results["fp64"]
        step_s = (r["ms_flow"] + r["ms_thermal"]) / 1e3
        tflops = FP64_FLOP_PER_CELL * cells / step_s / 1e12
        pk = fp64_peak_tflops()
        sm_mhz = clocks.get("sm_mhz") or 2070.0
        import torch
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        issue_peak = 2.0 * sms * sm_mhz * 1e6  # FP64 pipe: 2 thread instructions per clock per SM
        return {"bound": "fp64", "achieved": tflops, "peak": pk, "unit": "TFLOP/s", "frac": tflops / pk,
                "peak_kind": "measured live: cuBLAS DGEMM 8192^3", "flop_per_cell": FP64_FLOP_PER_CELL,
                "issue_frac": FP64_INST_PER_CELL * cells / step_s / issue_peak,
                "issue_peak_note": "FP64 pipe 2 thread instructions / clock / SM at the sampled SM clock"}

    head = results[precs[0]]
    line = {
        "metric": METRIC, "value": head["mlups"] * world, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPE[precs[0]], "data": "synthetic", "config": workload_config(args.size),
        "parallelism": "replicas" if world > 1 else "single GPU",
        "roofline": roof(precs[0]),
        "roofline_fp64": roof_fp64() if "fp64" in results else None,
        "e2e": e2e,
        "gpu_launches": LAUNCHES_PER_STEP[precs[0]] * args.steps,
        "clocks": clocks,
        "forms": {prec: {"mlups": results[prec]["mlups"] * world, "ms_per_step": results[prec]["ms_per_step"],
                         "dtype": DTYPE[prec], "roofline": roof(prec), "Nu": results[prec]["Nu"],
                         "Re": results[prec]["Re"]} for prec in results},
    }
    if rank == 0 and not args.no_128 and args.size != 128:
        leg = {}
        for prec in precs:
            r = time_precision(prec, args, None, local, size=128)
            leg[prec] = {"mlups": r["mlups"], "ms_per_step": r["ms_per_step"], "ms_flow": r["ms_flow"],
                         "ms_thermal": r["ms_thermal"], "Nu": r["Nu"], "Re": r["Re"],
                         "hbm_frac": BYTES_PER_CELL[prec] * 128 ** 3 / ((r["ms_flow"] + r["ms_thermal"]) / 1e3) / 1e9
                         / peak}
        line["cube128"] = {"workload": workload_config(128)["workload"], "forms": leg,
                               "note": "hbm_frac: algorithmic bytes over the flow + thermal kernel time per step, "
                                       "of the measured HBM peak"}
    if rank == 0 and not args.no_ensemble:
        line["batched"] = ensemble_run(args, local)
    if rank == 0 and not args.no_served:
        for prec in args.served_precisions.split(","):
            line["served" if prec == "fp32" else "served_" + prec] = served_run(args, local, prec)
    if rank == 0 and not args.no_size:
        line["at_384"] = at_size_run(args, local, peak)
    if rank == 0 and not args.no_rb2d:
        line["rb2d_256x128"] = rb2d_run(args, local)
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(n=args.size, device=local)
    if rank == 0:
        print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end (host buffers) leg")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched-form leg (64 2D instances)")
    ap.add_argument("--no-served", action="store_true", help="skip the served-stream leg")
    ap.add_argument("--no-size", action="store_true", help="skip the 384^3 leg (in-place vs two-buffer pattern)")
    ap.add_argument("--no-rb2d", action="store_true", help="skip the 2D 256 x 128 FP64 leg (20,000 steps)")
    ap.add_argument("--served-full", action="store_true", help="served leg as configured: 600 s, 5000-step window")
    ap.add_argument("--served-precisions", default="fp32,fp64x",
                    help="served legs: fp32 (batched form), fp64x (FP64 accuracy, one stream per solve)")
    ap.add_argument("--served-seconds", type=float, default=20.0)
    ap.add_argument("--served-drain", type=float, default=40.0)
    ap.add_argument("--served-window", type=int, default=1000)
    ap.add_argument("--served-cap", type=int, default=4000)
    ap.add_argument("--served-sample", type=int, default=10, help="served requests re-run one at a time in FP64")
    ap.add_argument("--served-plain-budget", type=float, default=90.0,
                    help="seconds for the one-at-a-time FP64 re-runs of the served sample")
    ap.add_argument("--size", type=int, default=N_CELL_EDGE, help="cube edge (cells); 256 is the benchmark")
    ap.add_argument("--precisions", default="fp64x,fp64,fp32,fp16",
                    help="comma list; the first is the headline form (fp64x: FP64 handle, fixed arithmetic)")
    ap.add_argument("--no-128", action="store_true", help="skip the 128^3 secondary leg")
    ap.add_argument("--accuracy", choices=["cube128", "cube384"], default=None,
                    help="instead of the benchmark: time-averaged Nu/Re of the storage forms against FP64")
    ap.add_argument("--accuracy-forms", default="fp64,fp64:1,fp32,fp32:1,fp16,fp16:1",
                    help="comma list of precision[:seed offset] runs of the accuracy leg")
    ap.add_argument("--accuracy-ref", default="fp64", help="precision of the run the others are compared with")
    ap.add_argument("--accuracy-steps", type=int, default=0, help="steps per run (0: the configuration's own)")
    ap.add_argument("--accuracy-every", type=int, default=500, help="steps between calNuRe samples")
    ap.add_argument("--accuracy-series", default=None, help="write the sampled (step, Nu, Re) series to this file")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.served_full:
        args.served_seconds, args.served_drain, args.served_window, args.served_cap = 600.0, 600.0, 5000, 50000
        args.served_plain_budget = max(args.served_plain_budget, 300.0)
    if args.impl == "reference":
        return run_reference(args)
    if args.accuracy:
        import torch
        torch.cuda.set_device(0)
        from lbmgpu import build as lbuild
        lbuild.build()
        return accuracy_run(args, 0)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
