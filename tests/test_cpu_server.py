"""The solve server's scheduling logic on the CPU, with stand-ins for the lattices.

The GPU tests run the server on the library; these check its policies without a GPU:
the windowed steady-Nu criterion, admission that passes over a request that does not fit
yet (and stops passing over it after `max_bypass` admissions), requests that fail to start
ending as rejected while the others run on, the step cap, and the summary's separation of
converged from capped solves."""
import math

import pytest

from lbmgpu.server import Request, SolveServer, summarize, windowed_steady


class FakeLattice:
    """A solve whose Nu relaxes towards nu_inf with time constant tau (in steps)."""

    def __init__(self, params, tau=1000.0, nu_inf=5.0, fail=False, osc=0.0):
        if fail:
            raise MemoryError("cudaMalloc refused")
        self.params = params
        self.itc = 0
        self.tau = tau
        self.nu_inf = nu_inf
        self.osc = osc  # amplitude of an oscillation that keeps the windowed mean moving
        self.closed = False

    def initial(self):
        self.itc = 0

    def calNuRe(self):
        nu = self.nu_inf - (self.nu_inf - 1.0) * math.exp(-self.itc / self.tau)
        return nu + self.osc * math.sin(self.itc / 1100.0), 10.0

    def close(self):
        self.closed = True


class FakeEnsemble:
    def __init__(self):
        self.members = []
        self.steps = 0

    def add(self, lat):
        self.members.append(lat)

    def remove(self, lat):
        self.members.remove(lat)

    def step(self, n):
        self.steps += n
        for m in self.members:
            m.itc += n

    def sync(self):
        pass

    def autotune(self, n):
        pass

    def close(self):
        pass


def make_server(budget=100, fail=(), tau=None, osc=None, **kw):
    """Footprint = the request's n (so budgets are easy to read); `fail`: rids whose lattice
    creation raises; `tau`: per-rid relaxation times; `osc`: per-rid oscillation amplitudes
    (a solve that never settles)."""
    tau = tau or {}
    osc = osc or {}
    created = []

    def factory(p):
        rid = p.seed - 1000
        lat = FakeLattice(p, tau=tau.get(rid, 500.0), fail=rid in fail, osc=osc.get(rid, 0.0))
        created.append((rid, lat))
        return lat

    srv = SolveServer(hbm_budget_bytes=budget, lattice_factory=factory, ensemble=FakeEnsemble(),
                      footprint_fn=lambda p: p.ny if p.dim == 2 else p.nx, **kw)
    return srv, created


def req(rid, n, arrival=0.0):
    return Request(rid, 2, n, 1e5, 0.71, 1000 + rid, arrival=arrival)


def test_windowed_criterion():
    flat = [(s, 4.0) for s in range(500, 10500, 500)]
    assert windowed_steady(flat, 5000, 1e-3)
    assert not windowed_steady(flat[:19], 5000, 1e-3)  # fewer than two windows
    drift = [(s, 4.0 + s * 1e-4) for s in range(500, 10500, 500)]
    assert not windowed_steady(drift, 5000, 1e-3)


def test_admission_passes_over_a_request_that_does_not_fit():
    srv, created = make_server(budget=100, chunk_steps=500, window=1000, max_steps=4000, max_bypass=8)
    # 60 runs; 50 does not fit beside it; 30 fits and is admitted ahead of 50
    results = srv.run([req(0, 60), req(1, 50), req(2, 30)])
    order = [rid for rid, _ in created]
    assert order.index(2) < order.index(1)
    assert {r.rid for r in results} == {0, 1, 2}
    assert all(r.steps > 0 for r in results)


def test_bypass_is_bounded():
    srv, created = make_server(budget=100, chunk_steps=500, window=1000, max_steps=4000, max_bypass=1,
                               osc={0: 1.0})
    # 0 runs long; 1 (60) cannot fit; 2 (20) is admitted ahead of it (one bypass); 3 (5)
    # would fit too but must now wait until 1 has run
    srv.run([req(0, 60), req(1, 60), req(2, 20), req(3, 5)])
    order = [rid for rid, _ in created]
    assert order.index(2) < order.index(1) < order.index(3)


def test_failed_start_is_rejected_and_others_run():
    srv, created = make_server(budget=100, chunk_steps=500, window=1000, max_steps=4000, fail={1})
    results = {r.rid: r for r in srv.run([req(0, 20), req(1, 20), req(2, 20)])}
    assert results[1].rejected and results[1].steps == 0
    assert results[0].steps > 0 and results[2].steps > 0
    assert srv.used == 0


def test_cap_and_summary():
    srv, _ = make_server(budget=100, chunk_steps=500, window=1000, max_steps=3000, osc={0: 1.0}, tau={1: 100.0})
    results = {r.rid: r for r in srv.run([req(0, 10), req(1, 10)])}
    assert results[0].capped and results[0].steps == 3000
    assert results[1].converged and not results[1].capped
    s = summarize(list(results.values()), 3600.0)
    assert s["converged"] == 1 and s["capped"] == 1 and s["converged_solves_per_hour"] == 1.0
    assert s["completed_solves_per_hour"] == 2.0


def test_cell_steps_count_unfinished_solves():
    # a solve that never settles is cut off by the time limit: its steps still count
    ticks = iter(range(1000))
    srv, _ = make_server(budget=100, chunk_steps=500, window=1000, max_steps=50000, osc={0: 1.0})
    results = srv.run([req(0, 10)], time_limit=5.5, clock=lambda: float(next(ticks)), sleep=lambda t: None)
    assert results == [] and srv.cell_steps > 0
    cells = req(0, 10).cells
    assert srv.cell_steps % (500 * cells) == 0
    s = summarize(results, 10.0, srv.cell_steps)
    assert s["aggregate_mlups"] == srv.cell_steps / 10.0 / 1e6


def test_oversized_and_foreign_precision_requests_are_rejected():
    srv, _ = make_server(budget=50, chunk_steps=500, window=1000, max_steps=2000)
    other = req(2, 10)
    other.precision = "fp16"
    results = {r.rid: r for r in srv.run([req(0, 80), req(1, 10), other])}
    assert "exceeds" in results[0].rejected
    assert "precision" in results[2].rejected
    assert results[1].steps > 0


def test_step_cap_must_be_a_whole_number_of_chunks():
    with pytest.raises(ValueError):
        make_server(chunk_steps=500, window=1000, max_steps=1234)


def test_stream_batch_steps_every_member():
    """The FP64 forms' batch: each member advances with its own step call per chunk."""
    from lbmgpu.server import StreamBatch

    class Steppable(FakeLattice):
        def step(self, n):
            self.itc += n

        def sync(self):
            pass

    created = []

    def factory(p):
        lat = Steppable(p, tau=100.0)
        created.append(lat)
        return lat

    srv = SolveServer(hbm_budget_bytes=100, lattice_factory=factory, ensemble=StreamBatch(),
                      footprint_fn=lambda p: p.ny, chunk_steps=500, window=1000, max_steps=4000, precision="fp64x")
    reqs = [req(0, 10), req(1, 20)]
    for q in reqs:
        q.precision = "fp64x"
    results = {r.rid: r for r in srv.run(reqs)}
    assert set(results) == {0, 1} and all(r.converged for r in results.values())
    assert srv.cell_steps == sum(results[r].steps * reqs[r].cells for r in results)
