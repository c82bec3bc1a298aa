"""The batched form (many lattices, one launch per stage) and the solve server.

* An ensemble of uneven 2D/3D lattices advanced together must give every member exactly
  the state it reaches when advanced alone (same per-cell arithmetic; only the tile table
  differs), under launch configurations that take the members with even nx one cell or two
  x-adjacent cells per thread.
* The autotuner advances the members by real steps and keeps them consistent.
* lbm_footprint matches what lbm_create takes from the device.
* The server gives each solve the same result alone and in a mix of concurrent solves.
"""
import numpy as np
import pytest

from lbmgpu import Ensemble, Lattice, LbmError, footprint
from lbmgpu.abi import rb_params

pytestmark = pytest.mark.gpu

MEMBERS = [
    dict(dim=2, nx=64, ny=32, Ra=1e5, Pr=0.71, seed=1),
    dict(dim=2, nx=96, ny=48, Ra=3e6, Pr=7.0, seed=2),
    dict(dim=3, nx=16, ny=16, nz=16, Ra=1e6, Pr=0.71, seed=3),
    dict(dim=2, nx=128, ny=64, Ra=2e4, Pr=0.71, seed=4),
    dict(dim=3, nx=20, ny=12, nz=10, Ra=5e5, Pr=7.0, seed=5),
    dict(dim=2, nx=75, ny=30, Ra=2e5, Pr=0.71, seed=6, periodic_x=False),  # odd nx: one cell per thread
    dict(dim=3, nx=15, ny=12, nz=9, Ra=5e5, Pr=0.71, seed=7),
    dict(dim=2, nx=70, ny=20, Ra=1e5, Pr=0.71, seed=8),  # rows not aligned with tiles
]

# launch configurations: (block, tile_cells, grid_per_sm, pairs); pairs bit 0 pairs the 2D
# members with even nx, bit 1 the 3D members
LAUNCHES = [(128, 1024, 8, 0), (128, 1024, 8, 1), (256, 2048, 4, 3), (128, 512, 16, 2)]


def make(m, precision="fp32"):
    p = rb_params(noise_amp=1e-3, precision=precision, **m)
    lat = Lattice(p)
    lat.initial()
    return lat


@pytest.mark.parametrize("launch", LAUNCHES)
@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_ensemble_matches_individual(precision, launch):
    ens = Ensemble()
    block, tile, grid, pairs = launch
    ens.configure(block=block, tile_cells=tile, grid_per_sm=grid, pairs=pairs)
    assert ens.launch() == {"block": block, "tile_cells": tile, "grid_per_sm": grid, "pairs": pairs}
    batched = [make(m, precision) for m in MEMBERS]
    for lat in batched:
        ens.add(lat)
    alone = [make(m, precision) for m in MEMBERS]
    for n, chunk in enumerate((1, 37, 64)):  # first steps, direct launches and graph replay
        ens.step(chunk)
        for lat in alone:
            # a new member takes its first step (from the module arrays) alone, then the chunk
            lat.step(chunk + 1 if n == 0 else chunk)
    ens.sync()
    for a, b in zip(batched, alone):
        assert a.itc == b.itc == 103
        for name in ("f", "g", "T", "u"):
            x, y = a.get_state(name), b.get_state(name)
            assert np.array_equal(x, y), (name, np.abs(x - y).max())
    # remove one member mid-run; the others continue unaffected
    ens.remove(batched[1])
    ens.step(10)
    for lat in alone:
        lat.step(10)
    for i in range(len(MEMBERS)):
        if i != 1:
            assert np.array_equal(batched[i].get_state("T"), alone[i].get_state("T"))
    ens.close()


def test_autotune_keeps_members_consistent():
    ens = Ensemble()
    batched = [make(m) for m in MEMBERS]
    for lat in batched:
        ens.add(lat)
    cfg = ens.autotune(2)
    assert cfg["block"] in (128, 256) and cfg["tile_cells"] % cfg["block"] == 0 and cfg["pairs"] in (0, 1, 2, 3)
    steps = batched[0].itc
    assert all(lat.itc == steps for lat in batched)
    alone = [make(m) for m in MEMBERS]
    for lat in alone:
        lat.step(steps)
    for a, b in zip(batched, alone):
        assert np.array_equal(a.get_state("T"), b.get_state("T"))
    ens.close()


def test_ensemble_rejects_fp64_and_duplicates():
    ens = Ensemble()
    for bad in ((64, 1024, 8, 1), (128, 1000, 8, 1), (128, 1024, 0, 1), (256, 1024, 8, 4)):
        with pytest.raises(LbmError):
            ens.configure(*bad)
    p = rb_params(dim=2, nx=32, ny=16, Ra=1e5)
    lat = Lattice(p)
    lat.initial()
    with pytest.raises(LbmError):
        ens.add(lat)
    lat2 = make(MEMBERS[0])
    ens.add(lat2)
    with pytest.raises(LbmError):
        ens.add(lat2)
    ens.close()


def test_footprint_matches_allocation():
    import torch
    for m, prec in ((MEMBERS[2], "fp32"), (MEMBERS[0], "fp16"), (dict(dim=3, n=40, Ra=1e6), "fp64")):
        p = rb_params(noise_amp=0.0, precision=prec, **m)
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        lat = Lattice(p)
        lat.initial()
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        used = free0 - free1
        est = footprint(p)
        # allocations round up to 2 MiB pages; the estimate must cover the arrays
        assert est <= used + 64 * 2 ** 20 and used <= est + 64 * 2 ** 20, (used, est)
        lat.close()


@pytest.mark.parametrize("precision", ["fp32", "fp64x"])
def test_server_result_same_alone_and_in_mix(precision):
    """FP32: the batched form; fp64x: FP64 accuracy with one stream per solve."""
    from lbmgpu.server import Request, SolveServer
    reqs = [Request(0, 2, 32, 2e5, 0.71, 11, arrival=0.0), Request(1, 3, 16, 1e6, 7.0, 12, arrival=0.0),
            Request(2, 2, 48, 5e4, 0.71, 13, arrival=0.05), Request(3, 3, 12, 3e5, 0.71, 14, arrival=0.1)]
    for q in reqs:
        q.precision = precision
    kw = dict(chunk_steps=200, check_every=1000, rel_tol=1e-3, max_steps=6000, precision=precision)
    srv = SolveServer(**kw)
    mixed = {r.rid: r for r in srv.run(reqs)}
    srv.close()
    assert len(mixed) == 4
    for req in reqs:
        solo = SolveServer(**kw)
        r = solo.run([Request(req.rid, req.dim, req.n, req.Ra, req.Pr, req.seed, arrival=0.0,
                              precision=precision)])[0]
        solo.close()
        m = mixed[req.rid]
        assert r.steps == m.steps and r.converged == m.converged
        assert r.Nu == m.Nu and r.Re == m.Re, (req.rid, r.Nu, m.Nu)


def test_bounded_wait_timeout_is_reported_and_the_handle_stays_usable():
    """Failure detection without a GPU fault: the staged kernels' bounded mbarrier wait, run
    on a barrier armed for bytes that no copy delivers (nothing in flight), gives up after a
    few thousand polls; the next sync reports LBM_ERR_TIMEOUT, clears the flag, and the
    handle keeps stepping."""
    import math
    from lbmgpu import LbmError, load_library
    from lbmgpu.abi import LBM_ERR_TIMEOUT
    p = rb_params(dim=3, n=16, Ra=1e6, noise_amp=1e-3, precision="fp32")
    lat = Lattice(p)
    lat.initial()
    lat.step(4)
    lat.sync()
    assert load_library().lbm_selftest_wait_timeout(lat._h, 1 << 12) == 0
    with pytest.raises(LbmError) as e:
        lat.sync()
    assert e.value.status == LBM_ERR_TIMEOUT
    lat.sync()  # the flag was cleared by the report
    lat.step(8)
    nu, re = lat.calNuRe()
    assert math.isfinite(nu) and math.isfinite(re)
    lat.close()
