#!/usr/bin/env python3
"""Benchmark of the coupled thermal MRT-LBM time step on GB300.

Workload: 3D Rayleigh-Benard cube, D3Q19 MRT flow + D3Q7 MRT temperature, 128^3 cells,
no-slip walls, adiabatic side walls, hot bottom (+0.5) / cold top (-0.5), Ra = 1e7,
Pr = 0.71, free-fall velocity U = 0.1, linear T + seeded 1e-3 noise.  A "step" is one
coupled (flow + thermal) time step over the whole lattice; MLUPS counts one coupled cell
update as one, as the reference's runtime print does (3DRB.F90:303-305).

Headline `value`: the plain method (FP64, the reference's arithmetic) through the fused
kernels, inputs resident in HBM.  The FP32 / FP16 storage forms of the same workload are
reported beside it.  `e2e` is the same metric through the C ABI with host buffers in the
reference's Fortran layout (state in, steps, T field and Nu/Re out).  `cpu_baseline` is
the C++ restatement of the reference's OpenMP CPU path timed on this host's cores; the GPU
then runs the same steps and the two temperature fields are compared bit for bit.

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
N_CELL_EDGE = 128
BYTES_PER_CELL = {"fp64": 416, "fp32": 208, "fp16": 104}  # populations read + written once
# FP64 work of the plain method per coupled cell update (3D), counted by ncu on the fused
# kernels (sass thread instructions, flow + thermal): dadd 398, dmul 103, dfma 57.  Products
# with exact powers of two run on the integer pipes and are not counted.
FP64_INST_PER_CELL = 398 + 103 + 57
FP64_FLOP_PER_CELL = 398 + 103 + 2 * 57
DTYPE = {"fp64": "f64", "fp32": "f32", "fp16": "f16-storage/f32-arith"}
FALLBACK_HBM_GBS = 6800.0


def workload_params(precision="fp64", n=N_CELL_EDGE):
    from lbmgpu.abi import rb_params
    return rb_params(dim=3, n=n, Ra=1e7, Pr=0.71, U=0.1, noise_amp=1e-3, seed=20261203, precision=precision)


def workload_config(n=N_CELL_EDGE):
    return {
        "workload": "3D Rayleigh-Benard cube D3Q19/D3Q7 MRT, %d^3 cells, Ra=1e7, Pr=0.71, U=0.1, no-slip walls, "
                    "adiabatic sides, T linear + 1e-3 seeded noise (seed 20261203)" % n,
        "cells": n ** 3,
        "l2": "inputs larger than L2 (FP64 populations 872 MB, FP32 436 MB, FP16 218 MB per step)",
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


def time_precision(prec, args, pg, local):
    import torch
    import lbmgpu
    p = workload_params(prec, args.size)
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


def e2e_run(prec, args, local):
    """State in from host arrays (Fortran layout), K steps, T field and Nu/Re out, via the C ABI."""
    import numpy as np
    import lbmgpu
    p = workload_params(prec, args.size)
    lat = lbmgpu.Lattice(p, device=local)
    lat.initial()
    names = ["f", "g", "rho", "u", "v", "w", "T", "Bx_prev", "By_prev", "Bz_prev"]
    host = {k: np.ascontiguousarray(lat.get_state(k)) for k in names}
    lat.step(args.warmup)
    lat.sync()
    t0 = time.perf_counter()
    for k in names:
        lat.set_state(k, host[k])
    lat.step(args.steps)
    T = lat.get_state("T")
    nu, re = lat.calNuRe()
    dt = time.perf_counter() - t0
    lat.close()
    h2d = sum(a.nbytes for a in host.values())
    d2h = T.nbytes + 16
    cells = p.nx * p.ny * p.nz
    return {"value": cells * args.steps / dt / 1e6, "unit": UNIT, "h2d_bytes_per_step": h2d / args.steps,
            "d2h_bytes_per_step": d2h / args.steps,
            "job": "lbm_set_state x%d (Fortran-layout host arrays) + lbm_step(%d) + lbm_get_state(T) + lbm_calNuRe"
                   % (len(names), args.steps)}


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


def ensemble_run(args, local, steps_total=13000):
    """Batched form (BASELINE config 3): 64 D2Q9/D2Q5 RB instances, aspect 2, ny drawn from
    {64,...,512}, Ra log-uniform in [1e4, 1e8], Pr in {0.71, 7}, U = 0.1, FP32 storage, one
    launch per stage over a packed tile table, graph replay, autotuned tiles.  |dNu| is
    measured against FP64 plain solves of the four smallest instances."""
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
    # run on to a developed flow and compare the four smallest instances with FP64 solves
    done = lats[0].itc
    if steps_total > done:
        ens.step(steps_total - done)
    ens.sync()
    diverged = []
    nus = {}
    for m, lat in enumerate(lats):
        try:
            nus[m] = lat.calNuRe()[0]
        except lbmgpu.LbmDiverged:
            diverged.append({"ny": specs[m]["ny"], "Ra": specs[m]["Ra"], "Pr": specs[m]["Pr"],
                             "tauf": lat.constants()["tauf"]})
    small = sorted(nus, key=lambda m: (specs[m]["ny"], m))[:4]
    dnu = []
    for m in small:
        nu32 = nus[m]
        ref = lbmgpu.Lattice(rb_params(precision="fp64", **specs[m]), device=local)
        ref.initial()
        ref.step(lats[m].itc)
        nu64, _ = ref.calNuRe()
        ref.close()
        dnu.append({"ny": specs[m]["ny"], "Ra": specs[m]["Ra"], "Pr": specs[m]["Pr"], "steps": lats[m].itc,
                    "Nu_fp32_batched": nu32, "Nu_fp64_plain": nu64, "rel_dNu": abs(nu32 - nu64) / abs(nu64)})
    ens.close()
    for lat in lats:
        lat.close()
    return {"workload": "64 D2Q9/D2Q5 RB instances, aspect 2, ny in {64..512}, Ra log-uniform 1e4..1e8, "
                        "Pr in {0.71,7}, FP32 storage, %d cells" % cells,
            "aggregate_mlups": mlups, "ms_per_step": ms / k, "steps_timed": k, "autotuned": cfg,
            "launches_per_step": 2, "dNu_vs_fp64": dnu,
            "diverged": {"count": len(diverged), "cases": diverged,
                         "note": "under-resolved draws (tau_f close to 1/2) reported as LBM_ERR_DIVERGED"}}


def served_run(args, local, plain3d_mlups):
    """Served form (BASELINE config 4): Poisson arrivals at 2/s, half 2D (ny 64..512, aspect 2)
    half 3D (n 64..192), Ra log-uniform 1e4..1e8, Pr in {0.71, 7}, FP32, admission by an 80%
    HBM budget, each solve run until Nu changes by < 0.1% over a window of steps or a step cap.
    The default run is scaled to fit a bench (20 s of arrivals, 1000-step window, 4000-step
    cap); --served-full runs the configuration as stated (600 s, 5000-step window)."""
    import lbmgpu
    from lbmgpu import server as srv
    duration, drain = args.served_seconds, args.served_drain
    window, cap = args.served_window, args.served_cap
    reqs = srv.poisson_requests(2.0, duration)
    s = srv.SolveServer(device=local, chunk_steps=500, check_every=window, rel_tol=1e-3, max_steps=cap,
                        autotune=False)
    t0 = time.perf_counter()
    results = s.run(reqs, time_limit=duration + drain)
    wall = time.perf_counter() - t0
    unfinished = len(s.active) + len(s.queue) + (len(reqs) - len(results) - len(s.active) - len(s.queue))
    summary = srv.summarize(results, wall)
    peak = (s.peak_active, s.peak_queue)
    s.close()
    # plain FP64 method, one solve at a time, on the same completed work
    plain2d = plain_rate_2d(local)
    by_id = {r.rid: r for r in reqs}
    done = [r for r in results if r.steps > 0]
    plain_s = sum(r.cells * r.steps / ((plain2d if by_id[r.rid].dim == 2 else plain3d_mlups) * 1e6) for r in done)
    # |dNu| of the two smallest completed solves against FP64 plain solves of the same length
    dnu = []
    for r in sorted([r for r in done if not r.diverged], key=lambda r: r.cells)[:2]:
        q = by_id[r.rid]
        p64 = q.params()
        p64.precision = 0
        ref = lbmgpu.Lattice(p64, device=local)
        ref.initial()
        ref.step(r.steps)
        nu64, _ = ref.calNuRe()
        ref.close()
        dnu.append({"rid": r.rid, "dim": q.dim, "n": q.n, "Ra": q.Ra, "steps": r.steps, "Nu_fp32_served": r.Nu,
                    "Nu_fp64_plain": nu64, "rel_dNu": abs(r.Nu - nu64) / abs(nu64)})
    summary.update({
        "workload": "Poisson arrivals 2/s for %.0f s, 50/50 2D (ny 64..512, aspect 2) / 3D (n 64..192), Ra "
                    "log-uniform 1e4..1e8, Pr {0.71,7}, FP32, 80%% HBM budget, stop at |dNu|<0.1%% over %d steps or "
                    "at %d steps; drain limit %.0f s%s" % (duration, window, cap, drain,
                    "" if args.served_full else " (scaled from 600 s / 5000-step window: the stated stream "
                    "oversubscribes one GPU several times)"),
        "arrived": len(reqs), "unfinished_at_limit": unfinished, "wall_s": wall,
        "peak_active": peak[0], "peak_queue": peak[1],
        "plain_fp64_solves_per_hour_same_work": 3600.0 * len(done) / plain_s if plain_s > 0 else None,
        "dNu_vs_fp64": dnu,
    })
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


def config0_run(args, local, steps=20000, cpu_steps=20000):
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
        "gpu_launches": 2 * args.steps,
        "clocks": clocks,
        "forms": {prec: {"mlups": results[prec]["mlups"] * world, "ms_per_step": results[prec]["ms_per_step"],
                         "dtype": DTYPE[prec], "roofline": roof(prec), "Nu": results[prec]["Nu"],
                         "Re": results[prec]["Re"]} for prec in results},
    }
    if rank == 0 and not args.no_ensemble:
        line["batched"] = ensemble_run(args, local)
    if rank == 0 and not args.no_served:
        line["served"] = served_run(args, local, results["fp64"]["mlups"] if "fp64" in results else 700.0)
    if rank == 0 and not args.no_size:
        line["at_384"] = at_size_run(args, local, peak)
    if rank == 0 and not args.no_config0:
        line["config0_2d"] = config0_run(args, local)
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
    ap.add_argument("--no-config0", action="store_true", help="skip the 2D 256 x 128 FP64 leg (20,000 steps)")
    ap.add_argument("--served-full", action="store_true", help="served leg as configured: 600 s, 5000-step window")
    ap.add_argument("--served-seconds", type=float, default=20.0)
    ap.add_argument("--served-drain", type=float, default=40.0)
    ap.add_argument("--served-window", type=int, default=1000)
    ap.add_argument("--served-cap", type=int, default=4000)
    ap.add_argument("--size", type=int, default=N_CELL_EDGE, help="cube edge (cells); 128 is the benchmark")
    ap.add_argument("--precisions", default="fp64,fp32,fp16",
                    help="comma list; the first is the headline form")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.served_full:
        args.served_seconds, args.served_drain, args.served_window, args.served_cap = 600.0, 1200.0, 5000, 50000
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
