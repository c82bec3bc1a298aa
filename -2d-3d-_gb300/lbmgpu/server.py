"""Continuous-batching solve server on top of the batched form.

Requests (a Rayleigh-Benard solve each: 2D or 3D, size, Ra, Pr, seed) arrive over time.
The server keeps every admitted lattice resident in HBM and advances all of them together
with one flow and one thermal launch per step (lbm_ensemble_step).  A request is admitted
as soon as its device footprint (lbm_footprint) fits under the HBM budget, so requests
that arrive while others are running join the running batch at the next chunk boundary.
Each solve runs until its volume Nusselt number (calNuRe, 2DRB.F90:1610-1675) changes by
less than `rel_tol` over `check_every` steps, or until `max_steps`.  Per-solve arithmetic
does not depend on which other lattices share the launches, so a result is the same alone
and in the mix.
"""
import heapq
import math
import time
from dataclasses import dataclass, field

from . import Ensemble, Lattice, LbmDiverged, footprint
from .abi import rb_params


@dataclass
class Request:
    rid: int
    dim: int
    n: int                 # 3D cube edge, or ny in 2D (nx = 2 ny)
    Ra: float
    Pr: float
    seed: int
    arrival: float = 0.0   # seconds after the start of the run
    precision: str = "fp32"

    def params(self):
        if self.dim == 2:
            return rb_params(dim=2, ny=self.n, nx=2 * self.n, Ra=self.Ra, Pr=self.Pr, U=0.1, noise_amp=1e-3,
                             seed=self.seed, precision=self.precision)
        return rb_params(dim=3, n=self.n, Ra=self.Ra, Pr=self.Pr, U=0.1, noise_amp=1e-3, seed=self.seed,
                         precision=self.precision)

    @property
    def cells(self):
        return 2 * self.n * self.n if self.dim == 2 else self.n ** 3


@dataclass
class Result:
    rid: int
    Nu: float
    Re: float
    steps: int
    converged: bool
    arrival: float
    admitted: float
    finished: float
    cells: int
    nu_history: list = field(default_factory=list)
    diverged: bool = False

    @property
    def time_to_solution(self):
        return self.finished - self.arrival


def poisson_requests(rate, duration, seed=20261203, sizes_2d=(64, 96, 128, 192, 256, 384, 512),
                     sizes_3d=(64, 96, 128, 160, 192), ra_range=(1e4, 1e8), prandtl=(0.71, 7.0)):
    """Poisson arrivals at `rate` per second for `duration` seconds; half 2D, half 3D."""
    import random
    rng = random.Random(seed)
    t, rid, out = 0.0, 0, []
    while True:
        t += rng.expovariate(rate)
        if t >= duration:
            break
        dim = 2 if rng.random() < 0.5 else 3
        n = rng.choice(sizes_2d if dim == 2 else sizes_3d)
        ra = math.exp(rng.uniform(math.log(ra_range[0]), math.log(ra_range[1])))
        out.append(Request(rid, dim, n, ra, rng.choice(prandtl), seed + rid, arrival=t))
        rid += 1
    return out


class SolveServer:
    def __init__(self, device=0, hbm_budget_bytes=None, budget_fraction=0.8, chunk_steps=500, check_every=5000,
                 rel_tol=1e-3, max_steps=50000, autotune=False):
        if check_every % chunk_steps:
            raise ValueError("check_every must be a multiple of chunk_steps")
        self.device = device
        self.ens = Ensemble(device)
        if hbm_budget_bytes is None:
            import torch
            free, total = torch.cuda.mem_get_info(device)
            hbm_budget_bytes = int(total * budget_fraction)
        self.budget = int(hbm_budget_bytes)
        self.chunk = int(chunk_steps)
        self.check_every = int(check_every)
        self.rel_tol = float(rel_tol)
        self.max_steps = int(max_steps)
        self.autotune = autotune
        self.used = 0
        self.active = {}   # rid -> (request, lattice, bytes, admitted_t, last_check_nu, history)
        self.queue = []    # FIFO of waiting requests
        self.results = []
        self.peak_active = 0
        self.peak_queue = 0

    def _admit(self, now):
        admitted = False
        while self.queue:
            req = self.queue[0]
            need = footprint(req.params())
            if need > self.budget:
                self.queue.pop(0)  # can never fit: reject
                self.results.append(Result(req.rid, float("nan"), float("nan"), 0, False, req.arrival, now, now,
                                           req.cells))
                continue
            if self.used + need > self.budget:
                break
            self.queue.pop(0)
            lat = Lattice(req.params(), device=self.device)
            lat.initial()
            self.ens.add(lat)
            self.used += need
            self.active[req.rid] = [req, lat, need, now, None, []]
            admitted = True
        self.peak_active = max(self.peak_active, len(self.active))
        return admitted

    def _finish(self, rid, now, converged, nu, re, diverged=False):
        req, lat, need, adm, _, hist = self.active.pop(rid)
        self.results.append(Result(rid, nu, re, lat.itc, converged, req.arrival, adm, now, req.cells, hist,
                                   diverged))
        self.ens.remove(lat)
        lat.close()
        self.used -= need

    def _check(self, now):
        for rid in list(self.active):
            req, lat, need, adm, last, hist = self.active[rid]
            steps = lat.itc
            due = steps >= (len(hist) + 1) * self.check_every
            if not due and steps < self.max_steps:
                continue
            try:
                nu, re = lat.calNuRe()
            except LbmDiverged:
                # non-finite field or rho <= 0: end this solve, keep serving the others
                self._finish(rid, now, False, float("nan"), float("nan"), diverged=True)
                continue
            hist.append((steps, nu))
            if last is not None and abs(nu - last) <= self.rel_tol * abs(last):
                self._finish(rid, now, True, nu, re)
            elif steps >= self.max_steps:
                self._finish(rid, now, False, nu, re)
            else:
                self.active[rid][4] = nu

    def run(self, requests, time_limit=None, clock=time.perf_counter):
        """Serve `requests` (arrival times relative to the start); returns the results."""
        pending = sorted(requests, key=lambda r: r.arrival)
        t0 = clock()
        i = 0
        tuned = False
        while i < len(pending) or self.queue or self.active:
            now = clock() - t0
            if time_limit is not None and now > time_limit:
                break
            while i < len(pending) and pending[i].arrival <= now:
                self.queue.append(pending[i])
                i += 1
            self.peak_queue = max(self.peak_queue, len(self.queue))
            self._admit(now)
            if not self.active:
                if i < len(pending):
                    time.sleep(max(0.0, min(0.05, pending[i].arrival - now)))
                continue
            if self.autotune and not tuned and len(self.active) > 1:
                self.ens.autotune(2)
                tuned = True
            self.ens.step(self.chunk)
            self.ens.sync()
            self._check(clock() - t0)
        return self.results

    def close(self):
        for rid in list(self.active):
            req, lat, need, adm, last, hist = self.active.pop(rid)
            self.ens.remove(lat)
            lat.close()
        self.ens.close()


def summarize(results, wall_seconds):
    done = [r for r in results if r.steps > 0]
    tts = sorted(r.time_to_solution for r in done)

    def pct(p):
        if not tts:
            return None
        k = min(len(tts) - 1, max(0, int(math.ceil(p / 100.0 * len(tts))) - 1))
        return tts[k]

    cells_steps = sum(r.cells * r.steps for r in done)
    return {
        "completed": len(done),
        "converged": sum(1 for r in done if r.converged),
        "capped": sum(1 for r in done if not r.converged and not r.diverged),
        "diverged": sum(1 for r in done if r.diverged),
        "solves_per_hour": 3600.0 * len(done) / wall_seconds if wall_seconds > 0 else None,
        "p50_s": pct(50),
        "p99_s": pct(99),
        "aggregate_mlups": cells_steps / wall_seconds / 1e6 if wall_seconds > 0 else None,
    }
