"""The in-place (AA) access pattern against the two-buffer (A/B) pattern and the oracle.

One population array per lattice, whose layout alternates between the streamed and the
swapped form, must give the same values as the two-buffer step, bit for bit, for every
storage precision and every boundary kind: walls (bounce-back, constant-T, adiabatic)
are resolved inside a cell, and a periodic face is crossed through a snapshot of the face
slots taken before each odd sweep.  State transfer, restart files and the CUDA-graph
chunks see the layout through the same rules."""
import os

import numpy as np
import pytest

from lbmgpu import Ensemble, LbmError, Lattice
from lbmgpu.abi import (FIELDS, LBM_BC_PERIODIC, LBM_BCT_ADIABATIC, LBM_BCT_CONST, LBM_BCT_PERIODIC, LBM_CELL_SIDE,
                        field_shape, rb_params)

pytestmark = pytest.mark.gpu


def cases():
    out = {
        "2d_periodic_x": rb_params(dim=2, nx=40, ny=20, Ra=1e5, noise_amp=1e-3, seed=31),
        "2d_walls": rb_params(dim=2, nx=36, ny=18, Ra=2e5, noise_amp=1e-3, seed=32, periodic_x=False),
        "3d_noslip": rb_params(dim=3, nx=16, ny=14, nz=12, Ra=1e6, noise_amp=1e-3, seed=33),
        "3d_periodic_xz": rb_params(dim=3, nx=14, ny=10, nz=8, Ra=1e6, noise_amp=1e-3, seed=34, periodic_x=True),
        "3d_odd": rb_params(dim=3, nx=13, ny=9, nz=7, Ra=1e6, noise_amp=1e-3, seed=35),
        "3d_legacy_periodic_z": rb_params(dim=3, nx=12, ny=10, nz=8, Ra=1e5, U=0.02, noise_amp=1e-3, seed=36,
                                          legacy_thermal=True),
    }
    p = out["3d_periodic_xz"]
    p.bc_flow[2] = LBM_BC_PERIODIC
    p.bc_thermal[2] = LBM_BCT_PERIODIC
    p = out["3d_legacy_periodic_z"]
    p.bc_flow[2] = LBM_BC_PERIODIC
    p.bc_thermal[2] = LBM_BCT_PERIODIC
    side = rb_params(dim=3, nx=12, ny=10, nz=6, Ra=1e5, noise_amp=1e-3, seed=37)
    side.cell = LBM_CELL_SIDE
    side.bc_thermal[0] = LBM_BCT_CONST
    side.bc_thermal[1] = LBM_BCT_ADIABATIC
    out["3d_side_heated"] = side
    side2 = rb_params(dim=2, nx=24, ny=24, Ra=1e5, noise_amp=1e-3, seed=38, periodic_x=False)
    side2.cell = LBM_CELL_SIDE
    side2.bc_thermal[0] = LBM_BCT_CONST
    side2.bc_thermal[1] = LBM_BCT_ADIABATIC
    out["2d_side_heated"] = side2
    return out


def fields(p):
    names = ["f", "g", "rho", "u", "v", "T", "Bx_prev", "By_prev"]
    names += ["w", "Bz_prev"] if p.dim == 3 else ["Fy"]
    return names


def pair(p):
    a, b = p.copy(), p.copy()
    a.pattern, b.pattern = 1, 0
    return Lattice(a), Lattice(b)


def assert_same(aa, ab, p, tag):
    for name in fields(p):
        x, y = aa.get_state(name), ab.get_state(name)
        assert np.array_equal(x, y), (tag, name, float(np.nanmax(np.abs(x - y))))


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp16"])
@pytest.mark.parametrize("name", sorted(cases()))
def test_in_place_equals_two_buffers(name, precision):
    """Odd and even step counts, single steps and graph chunks, the state read back
    (module view of each layout) in between."""
    p = cases()[name].copy()
    p.precision = {"fp64": 0, "fp32": 1, "fp16": 2}[precision]
    aa, ab = pair(p)
    for lat in (aa, ab):
        lat.initial()
    done = 0
    for n in (1, 2, 5, 33, 64, 3):
        for lat in (aa, ab):
            lat.step(n)
        done += n
        assert_same(aa, ab, p, "%s %s after %d steps" % (name, precision, done))
    nu_a, re_a = aa.calNuRe()
    nu_b, re_b = ab.calNuRe()
    assert (nu_a, re_a) == (nu_b, re_b)


def test_in_place_magnetic_force():
    """SideHeatedHa (2D plain method) in the in-place pattern."""
    p = cases()["2d_side_heated"].copy()
    p.side_heated_ha, p.Ha, p.phi_deg = 1, 20.0, 30.0
    aa, ab = pair(p)
    for lat in (aa, ab):
        lat.initial()
        lat.step(41)
    assert_same(aa, ab, p, "Ha")


@pytest.mark.parametrize("dim", [2, 3])
def test_in_place_fp64_equals_oracle(oracle_mod, dim):
    """The plain method in the in-place pattern is bitwise the reference's CPU arithmetic."""
    p = rb_params(dim=2, nx=32, ny=16, Ra=1e5, noise_amp=1e-3, pattern="AA") if dim == 2 else \
        rb_params(dim=3, nx=10, ny=9, nz=8, Ra=1e6, noise_amp=1e-3, pattern="AA")
    g = Lattice(p)
    g.initial()
    g.step(37)
    o = oracle_mod.Oracle(p)
    o.initial()
    o.step(37)
    for name in ("f", "g", "T", "u", "v", "rho"):
        a = g.get_state(name)
        b = o.get(FIELDS[name], field_shape(p, name))
        assert np.array_equal(a, b), (dim, name, float(np.abs(a - b).max()))


@pytest.mark.parametrize("precision", ["fp64", "fp16"])
def test_in_place_state_loads_between_steps(precision):
    """Populations loaded while the array is in the swapped layout (the two arrays then
    run with different parities), and a module scalar loaded mid-run (first step again)."""
    p = cases()["3d_periodic_xz"].copy()
    p.precision = {"fp64": 0, "fp16": 2}[precision]
    aa, ab = pair(p)
    for lat in (aa, ab):
        lat.initial()
        lat.step(3)  # odd: the in-place arrays are swapped
    f = ab.get_state("f")
    u = ab.get_state("u")
    for lat in (aa, ab):
        lat.set_state("f", f * (1.0 + 1e-6))
        lat.step(5)
    assert_same(aa, ab, p, "after f load")
    for lat in (aa, ab):
        lat.set_state("u", u)
        lat.step(40)  # crosses a chunk with the thermal array one layout ahead
    assert_same(aa, ab, p, "after u load")
    g = ab.get_state("g")
    for lat in (aa, ab):
        lat.set_state("g", g)
        lat.step(33)
    assert_same(aa, ab, p, "after g load")


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp16"])
def test_in_place_restart(tmp_path, precision):
    """Continuation records of an in-place handle restart bit for bit (from either
    layout); the reference's two records load into either pattern."""
    p = cases()["3d_periodic_xz"].copy()
    p.precision = {"fp64": 0, "fp32": 1, "fp16": 2}[precision]
    p.pattern = 1
    for stop in (6, 7):
        run = Lattice(p)
        run.initial()
        run.step(stop)
        path = os.path.join(str(tmp_path), "rst_%d.bin" % stop)
        run.backupData(path, continuation=True)
        run.step(20)
        again = Lattice(p)
        again.reload(path, mode="continue")
        again.step(20)
        for name in fields(p):
            assert np.array_equal(run.get_state(name), again.get_state(name)), (precision, stop, name)
    # the reference records only: same reconstruction in both patterns
    q = p.copy()
    q.pattern = 0
    a, b = Lattice(p), Lattice(q)
    a.reload(path, mode="reference")
    b.reload(path, mode="reference")
    for lat in (a, b):
        lat.step(9)
    assert_same(a, b, p, "reference reload")


def test_in_place_refusals():
    p = rb_params(dim=3, n=10, Ra=1e6, pattern="AA")
    lat = Lattice(p)
    lat.initial()
    lat.step(3)
    with pytest.raises(LbmError):
        lat.get_state("f_post")
    with pytest.raises(LbmError):
        lat.collision()  # the stage entry points need f and f_post
    q = p.copy()
    q.precision = 1
    fast = Lattice(q)
    fast.initial()
    ens = Ensemble()
    with pytest.raises(LbmError):
        ens.add(fast)


@pytest.mark.parametrize("pairs", [0, 1])
@pytest.mark.parametrize("precision", ["fp32", "fp16"])
@pytest.mark.parametrize("name", ["3d_periodic_xz", "3d_side_heated", "2d_walls", "2d_periodic_x"])
def test_in_place_forms(name, precision, pairs):
    """One cell per thread and two cells per thread in the in-place pattern, against the
    two-buffer default form."""
    from lbmgpu import LBM_OPT_PAIRS
    p = cases()[name].copy()
    p.precision = {"fp32": 1, "fp16": 2}[precision]
    aa, ab = pair(p)
    aa.set_option(LBM_OPT_PAIRS, pairs)
    for lat in (aa, ab):
        lat.initial()
        lat.step(69)
    assert_same(aa, ab, p, "%s %s pairs=%d" % (name, precision, pairs))


def staged_cases():
    """Lattices with nx a multiple of 8 (the staged kernels' rows are 16-byte aligned)."""
    out = {
        "noslip": rb_params(dim=3, nx=16, ny=14, nz=12, Ra=1e6, noise_amp=1e-3, seed=41),
        "periodic_xz": rb_params(dim=3, nx=16, ny=10, nz=8, Ra=1e6, noise_amp=1e-3, seed=42, periodic_x=True),
        "legacy_periodic_z": rb_params(dim=3, nx=24, ny=10, nz=8, Ra=1e5, U=0.02, noise_amp=1e-3, seed=43,
                                       legacy_thermal=True),
    }
    for name in ("periodic_xz", "legacy_periodic_z"):
        out[name].bc_flow[2] = LBM_BC_PERIODIC
        out[name].bc_thermal[2] = LBM_BCT_PERIODIC
    side = rb_params(dim=3, nx=16, ny=10, nz=6, Ra=1e5, noise_amp=1e-3, seed=44)
    side.cell = LBM_CELL_SIDE
    side.bc_thermal[0] = LBM_BCT_CONST
    side.bc_thermal[1] = LBM_BCT_ADIABATIC
    out["side_heated"] = side
    return out


@pytest.mark.parametrize("staged", [0, 1])
@pytest.mark.parametrize("precision", ["fp32", "fp16"])
@pytest.mark.parametrize("name", sorted(staged_cases()))
def test_in_place_staged(name, precision, staged):
    """Staged rows (bulk copies into shared memory) in the in-place pattern: interior tiles
    staged from the swapped or the streamed layout, face cells on the one-cell path."""
    from lbmgpu import LBM_OPT_STAGED
    p = staged_cases()[name].copy()
    p.precision = {"fp32": 1, "fp16": 2}[precision]
    aa, ab = pair(p)
    aa.set_option(LBM_OPT_STAGED, staged)
    for lat in (aa, ab):
        lat.initial()
    for n in (2, 35, 32, 1):
        for lat in (aa, ab):
            lat.step(n)
        assert_same(aa, ab, p, "%s %s staged=%d" % (name, precision, staged))
    aa.sync()


def test_in_place_staged_mixed_layouts():
    """After populations are loaded into one array only, the arrays' layouts are out of step
    and the staged sweeps give way to the one-cell kernels; results stay equal."""
    p = staged_cases()["periodic_xz"].copy()
    p.precision = 2
    aa, ab = pair(p)
    for lat in (aa, ab):
        lat.initial()
        lat.step(3)
    g = ab.get_state("g")
    for lat in (aa, ab):
        lat.set_state("g", g)
        lat.step(37)
    assert_same(aa, ab, p, "mixed layouts")
