"""Continuous-batching solve server on top of the batched form.

Requests (a Rayleigh-Benard solve each: 2D or 3D, size, Ra, Pr, seed) arrive over time.
The server keeps every admitted lattice resident in HBM and advances all of them together
with one flow and one thermal launch per step (lbm_ensemble_step) in FP32/FP16 storage, or,
for solves at FP64 accuracy (the fixed arithmetic, "fp64x", or the plain method, "fp64"),
each with its own lbm_step on its own stream so that their launches overlap.  Requests that arrive
while others run are admitted as soon as their device footprint (lbm_footprint) fits under
the HBM budget, and join the running batch at the next chunk boundary.

Admission walks the queue in arrival order and admits every request that fits, so a large
request that does not fit yet does not hold back smaller ones behind it.  The bypass is
bounded: once the oldest waiting request has been passed over `max_bypass` times, nothing
behind it is admitted until it fits, so it cannot starve.

Each solve samples its volume Nusselt number (calNuRe, 2DRB.F90:1610-1675) every chunk and
stops when the mean of the last `window` steps differs from the mean of the `window` steps
before by less than `rel_tol` (the windowed steady-Nu criterion; the reference's own
stopping test compares fields 2000 steps apart, 3DRB.F90:225, 245-247), at `max_steps`
(capped, reported apart from converged solves), or when a diagnostic reports divergence.
A request whose lattice cannot be created (device memory, parameters) ends as rejected
without stopping the others.  Per-solve arithmetic does not depend on which other lattices
share the launches, so a result is the same alone and in the mix.
"""
import math
import time
from dataclasses import dataclass, field

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

    def params(self, precision=None):
        prec = precision or self.precision
        if self.dim == 2:
            return rb_params(dim=2, ny=self.n, nx=2 * self.n, Ra=self.Ra, Pr=self.Pr, U=0.1, noise_amp=1e-3,
                             seed=self.seed, precision=prec)
        return rb_params(dim=3, n=self.n, Ra=self.Ra, Pr=self.Pr, U=0.1, noise_amp=1e-3, seed=self.seed,
                         precision=prec)

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
    rejected: str = ""     # why the request was not run ("" when it ran)

    @property
    def time_to_solution(self):
        return self.finished - self.arrival

    @property
    def capped(self):
        return self.steps > 0 and not self.converged and not self.diverged


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


def windowed_steady(history, window, rel_tol):
    """history: [(step, Nu)] sampled at a fixed stride.  True when the mean Nu of the last
    `window` steps differs from the mean of the `window` steps before it by less than
    rel_tol (relative to the latter)."""
    if len(history) < 2:
        return False
    stride = history[-1][0] - history[-2][0]
    if stride <= 0:
        return False
    k = max(1, window // stride)
    if len(history) < 2 * k:
        return False
    last = [nu for _, nu in history[-k:]]
    prev = [nu for _, nu in history[-2 * k:-k]]
    m1, m0 = sum(last) / k, sum(prev) / k
    return abs(m1 - m0) <= rel_tol * abs(m0)


class StreamBatch:
    """The ensemble interface for storage forms the batched kernels do not take (FP64: the
    plain method and the fixed arithmetic): every member advances with its own lbm_step on
    its own CUDA stream, so the members' launches overlap on the GPU.  A chunk is one
    lbm_step(n) per member, enqueued without waiting; sync waits for all of them."""

    def __init__(self):
        self.members = []

    def add(self, lat):
        self.members.append(lat)

    def remove(self, lat):
        self.members.remove(lat)

    def step(self, n):
        for lat in self.members:
            lat.step(n)

    def sync(self):
        for lat in self.members:
            lat.sync()

    def autotune(self, nsteps):
        pass

    def close(self):
        self.members = []


BATCHED_PRECISIONS = ("fp32", "fp16")


class SolveServer:
    """lattice_factory(params) -> a Lattice-like object (initial, calNuRe, itc, close);
    ensemble: an Ensemble-like object (add, remove, step, sync, autotune, close);
    footprint_fn(params) -> bytes.  The defaults are the library's own (the batched form for
    FP32/FP16, a StreamBatch for the FP64 forms "fp64" and "fp64x"); tests pass fakes."""

    def __init__(self, device=0, hbm_budget_bytes=None, budget_fraction=0.8, chunk_steps=500, window=5000,
                 rel_tol=1e-3, max_steps=50000, autotune=False, max_bypass=8, precision="fp32",
                 lattice_factory=None, ensemble=None, footprint_fn=None, check_every=None):
        if check_every is not None:  # older name of the window
            window = check_every
        if window % chunk_steps:
            raise ValueError("window must be a multiple of chunk_steps")
        if max_steps % chunk_steps:
            raise ValueError("max_steps must be a multiple of chunk_steps (the cap is checked between chunks)")
        self.device = device
        if lattice_factory is None or ensemble is None or footprint_fn is None:
            from . import Ensemble, Lattice, footprint
            lattice_factory = lattice_factory or (lambda p: Lattice(p, device=device))
            if ensemble is None:
                ensemble = Ensemble(device) if precision in BATCHED_PRECISIONS else StreamBatch()
            footprint_fn = footprint_fn or footprint
        self.make_lattice = lattice_factory
        self.ens = ensemble
        self.footprint = footprint_fn
        if hbm_budget_bytes is None:
            import torch
            free, total = torch.cuda.mem_get_info(device)
            # a fraction of the GPU, but never more than is free now (other users' memory)
            hbm_budget_bytes = int(min(total * budget_fraction, free * 0.95))
        self.budget = int(hbm_budget_bytes)
        self.precision = precision
        self.chunk = int(chunk_steps)
        self.window = int(window)
        self.rel_tol = float(rel_tol)
        self.max_steps = int(max_steps)
        self.autotune = autotune
        self.max_bypass = int(max_bypass)
        self.used = 0
        self.active = {}   # rid -> [request, lattice, bytes, admitted_t, history]
        self.queue = []    # waiting requests in arrival order
        self.bypassed = {}  # rid -> times a later request was admitted ahead of it
        self.results = []
        self.peak_active = 0
        self.peak_queue = 0
        self.cell_steps = 0  # cell updates advanced by the ensemble, finished solves or not

    def _reject(self, req, now, why):
        self.results.append(Result(req.rid, float("nan"), float("nan"), 0, False, req.arrival, now, now, req.cells,
                                   rejected=why))

    def _start(self, req, now, need):
        """Create, initialise and add one lattice; False (and a rejected result) on failure."""
        lat = None
        try:
            lat = self.make_lattice(req.params(self.precision))
            lat.initial()
            self.ens.add(lat)
        except Exception as e:  # device memory, parameters, ensemble refusal: this request only
            if lat is not None:
                try:
                    lat.close()
                except Exception:
                    pass
            self._reject(req, now, "%s: %s" % (type(e).__name__, e))
            return False
        self.used += need
        self.active[req.rid] = [req, lat, need, now, []]
        return True

    def _admit(self, now):
        admitted = False
        keep = []
        blocked = False  # the oldest waiting request has been bypassed max_bypass times
        for req in self.queue:
            try:
                need = self.footprint(req.params(self.precision))
            except Exception as e:
                self._reject(req, now, "parameters: %s" % e)
                continue
            if need > self.budget:
                self._reject(req, now, "footprint %d B exceeds the budget %d B" % (need, self.budget))
                continue
            if blocked or self.used + need > self.budget:
                keep.append(req)
                if not blocked and self.bypassed.get(req.rid, 0) >= self.max_bypass:
                    blocked = True
                continue
            if self._start(req, now, need):
                admitted = True
                for w in keep:  # everyone still waiting ahead of it was bypassed once more
                    self.bypassed[w.rid] = self.bypassed.get(w.rid, 0) + 1
                    if self.bypassed[w.rid] >= self.max_bypass:
                        blocked = True
        self.queue = keep
        self.peak_active = max(self.peak_active, len(self.active))
        return admitted

    def _finish(self, rid, now, converged, nu, re, diverged=False):
        req, lat, need, adm, hist = self.active.pop(rid)
        self.results.append(Result(rid, nu, re, lat.itc, converged, req.arrival, adm, now, req.cells, hist, diverged))
        self.ens.remove(lat)
        lat.close()
        self.used -= need
        self.bypassed.pop(rid, None)

    def _check(self, now):
        from . import LbmDiverged
        for rid in list(self.active):
            req, lat, need, adm, hist = self.active[rid]
            steps = lat.itc
            try:
                nu, re = lat.calNuRe()
            except LbmDiverged:
                # non-finite field or rho <= 0: end this solve, keep serving the others
                self._finish(rid, now, False, float("nan"), float("nan"), diverged=True)
                continue
            hist.append((steps, nu))
            if windowed_steady(hist, self.window, self.rel_tol):
                self._finish(rid, now, True, nu, re)
            elif steps >= self.max_steps:
                self._finish(rid, now, False, nu, re)

    def run(self, requests, time_limit=None, clock=time.perf_counter, sleep=time.sleep):
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
                if pending[i].precision != self.precision and pending[i].precision is not None:
                    self._reject(pending[i], now, "precision %s: this server batches %s" %
                                 (pending[i].precision, self.precision))
                else:
                    self.queue.append(pending[i])
                i += 1
            self.peak_queue = max(self.peak_queue, len(self.queue))
            self._admit(now)
            if not self.active:
                if i < len(pending):
                    sleep(max(0.0, min(0.05, pending[i].arrival - now)))
                elif self.queue:
                    break  # nothing running and nothing that fits: cannot happen with rejections above
                continue
            if self.autotune and not tuned and len(self.active) > 1:
                self.ens.autotune(2)
                tuned = True
            self.cell_steps += self.chunk * sum(a[0].cells for a in self.active.values())
            self.ens.step(self.chunk)
            self.ens.sync()
            self._check(clock() - t0)
        return self.results

    def close(self):
        for rid in list(self.active):
            req, lat, need, adm, hist = self.active.pop(rid)
            self.ens.remove(lat)
            lat.close()
        self.ens.close()


def summarize(results, wall_seconds, cell_steps=None):
    """cell_steps: every cell update the server advanced (SolveServer.cell_steps), including
    solves still running at a time limit; without it the aggregate counts finished solves."""
    ran = [r for r in results if r.steps > 0]
    conv = [r for r in ran if r.converged]
    tts = sorted(r.time_to_solution for r in conv)

    def pct(xs, p):
        if not xs:
            return None
        k = min(len(xs) - 1, max(0, int(math.ceil(p / 100.0 * len(xs))) - 1))
        return xs[k]

    tts_all = sorted(r.time_to_solution for r in ran)
    cells_steps = cell_steps if cell_steps is not None else sum(r.cells * r.steps for r in ran)
    return {
        "completed": len(ran),
        "converged": len(conv),
        "capped": sum(1 for r in ran if r.capped),
        "diverged": sum(1 for r in ran if r.diverged),
        "rejected": sum(1 for r in results if r.rejected),
        "converged_solves_per_hour": 3600.0 * len(conv) / wall_seconds if wall_seconds > 0 else None,
        "completed_solves_per_hour": 3600.0 * len(ran) / wall_seconds if wall_seconds > 0 else None,
        "p50_s": pct(tts, 50),
        "p99_s": pct(tts, 99),
        "p50_s_all_completed": pct(tts_all, 50),
        "p99_s_all_completed": pct(tts_all, 99),
        "aggregate_mlups": cells_steps / wall_seconds / 1e6 if wall_seconds > 0 else None,
    }
