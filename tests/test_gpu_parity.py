"""GPU parity: the CUDA kernels (through the C ABI) against the CPU oracle.

Plain FP64 method: every stage kernel and the fused step must reproduce the oracle bit for
bit (same operations in the same order, no FMA contraction, IEEE division); the required
bar is <= 1e-12 relative in the populations after 1000 steps and <= 1e-10 in Nu.
"""
import numpy as np
import pytest

from lbmgpu import Lattice, LbmError, LbmDiverged
from lbmgpu.abi import (FIELDS, LBM_BC_PERIODIC, LBM_BCT_ADIABATIC, LBM_BCT_CONST, LBM_BCT_PERIODIC, LBM_CELL_SIDE,
                        LbmNuWall, field_shape, rb_params)

pytestmark = pytest.mark.gpu

POP_RTOL = 1e-12   # populations after 1000 steps, relative to max |f|
NU_RTOL = 1e-10    # Nusselt / Reynolds numbers


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def pair(oracle_mod, p):
    o = oracle_mod.Oracle(p)
    o.initial()
    g = Lattice(p)
    g.initial()
    return o, g


def fields_for(p):
    names = ["f", "g", "rho", "u", "v", "T", "Bx_prev", "By_prev", "f_post", "g_post"]
    names += ["w", "Bz_prev"] if p.dim == 3 else ["Fx", "Fy"]
    return names


def assert_same(o, g, p, names=None, rtol=0.0):
    for name in names or fields_for(p):
        a = g.get_state(name)
        b = o.get(FIELDS[name], field_shape(p, name))
        if rtol == 0.0:
            assert np.array_equal(a, b), "%s differs: max |d| = %g" % (name, np.abs(a - b).max())
        else:
            assert rel_err(a, b) <= rtol, "%s rel err %g" % (name, rel_err(a, b))


CASES = {
    "2d_rb_periodic": dict(dim=2, nx=24, ny=12, Ra=1e5),
    "3d_rb_noslip": dict(dim=3, nx=10, ny=9, nz=8, Ra=1e6),
}


def make(case, **kw):
    args = dict(CASES[case])
    args.update(kw)
    return rb_params(noise_amp=1e-3, **args)


@pytest.mark.parametrize("case", list(CASES))
def test_initial_bitwise(oracle_mod, case):
    p = make(case)
    o, g = pair(oracle_mod, p)
    assert_same(o, g, p)


@pytest.mark.parametrize("case", list(CASES))
def test_stage_kernels_bitwise(oracle_mod, case):
    """Each of the eight stage kernels against the oracle's subroutine, three iterations."""
    p = make(case)
    o, g = pair(oracle_mod, p)
    stages = ["collision", "streaming", "bounceback", "macro", "collisionT", "streamingT", "bouncebackT", "macroT"]
    for _ in range(3):
        for s in stages:
            getattr(o, s)()
            getattr(g, s)()
            assert_same(o, g, p)


@pytest.mark.parametrize("case", list(CASES))
def test_fused_1000_steps(oracle_mod, case):
    p = make(case)
    o, g = pair(oracle_mod, p)
    o.step(1000)
    g.step(1000)
    for name in ("f", "g", "T", "u", "v", "rho"):
        a = g.get_state(name)
        b = o.get(FIELDS[name], field_shape(p, name))
        assert rel_err(a, b) <= POP_RTOL, (name, rel_err(a, b))
    # the plain method is bitwise identical to the oracle
    assert_same(o, g, p, ["f", "g", "T", "u", "v", "rho", "Bx_prev", "By_prev", "f_post", "g_post"])
    nu_o, re_o, _ = o.calNuRe()
    nu_g, re_g = g.calNuRe()
    assert nu_g == pytest.approx(nu_o, rel=NU_RTOL) and re_g == pytest.approx(re_o, rel=NU_RTOL)
    ng_o, _ = o.RBcalc_Nu_global()
    assert g.RBcalc_Nu_global() == pytest.approx(ng_o, rel=NU_RTOL)
    w_o, _ = o.RBcalc_Nu_wall_avg(LbmNuWall)
    w_g = g.RBcalc_Nu_wall_avg()
    for k, v in w_o.as_dict().items():
        assert w_g[k] == pytest.approx(v, rel=NU_RTOL, abs=1e-12), k
    eo = o.check()
    eg = g.check()
    assert eg[0] == pytest.approx(eo[0], rel=NU_RTOL) and eg[1] == pytest.approx(eo[1], rel=NU_RTOL)


def test_fused_and_stage_interleave(oracle_mod):
    """Fused steps, then stage kernels, then fused steps again stay on the oracle's trajectory."""
    p = make("3d_rb_noslip")
    o, g = pair(oracle_mod, p)
    g.step(7)
    for _ in range(3):
        g.stage_step()
    g.step(33)  # crosses a captured-graph chunk
    o.step(43)
    assert_same(o, g, p, ["f", "g", "T", "u", "v", "w", "rho", "Bx_prev", "By_prev", "Bz_prev"])
    assert g.itc == 43


VARIANTS = {
    "2d_legacy": dict(dim=2, nx=20, ny=10, Ra=1e5, legacy_thermal=True, U=0.05),
    "2d_no_m1g": dict(dim=2, nx=20, ny=10, Ra=1e5, use_g=False),
    "2d_small_ra_perturbed": dict(dim=2, nx=20, ny=10, Ra=5e3),
    "3d_small_ra_perturbed": dict(dim=3, nx=8, ny=8, nz=6, Ra=1e4),
    "3d_x_periodic": dict(dim=3, nx=8, ny=8, nz=6, Ra=1e6, periodic_x=True),
    "3d_legacy": dict(dim=3, nx=8, ny=8, nz=6, Ra=1e5, legacy_thermal=True, U=0.02),
}


@pytest.mark.parametrize("name", list(VARIANTS))
def test_variants_bitwise(oracle_mod, name):
    p = rb_params(noise_amp=1e-3, **VARIANTS[name])
    o, g = pair(oracle_mod, p)
    o.step(200)
    g.step(200)
    assert_same(o, g, p, ["f", "g", "T", "u", "v", "rho"])


def test_z_periodic_and_side_heated(oracle_mod):
    p = rb_params(dim=3, nx=8, ny=8, nz=6, Ra=1e5, noise_amp=1e-3)
    p.bc_flow[2] = LBM_BC_PERIODIC
    p.bc_thermal[2] = LBM_BCT_PERIODIC
    o, g = pair(oracle_mod, p)
    o.step(100)
    g.step(100)
    assert_same(o, g, p, ["f", "g", "T"])
    # side-heated cavity: hot/cold x walls, adiabatic y/z walls (3DRB.F90 default switches)
    p = rb_params(dim=3, nx=8, ny=8, nz=6, Ra=1e5, noise_amp=0.0)
    p.cell = LBM_CELL_SIDE
    p.bc_thermal[0] = LBM_BCT_CONST
    p.bc_thermal[1] = LBM_BCT_ADIABATIC
    o, g = pair(oracle_mod, p)
    o.step(100)
    g.step(100)
    assert_same(o, g, p, ["f", "g", "T"])
    assert g.calNuRe()[0] == pytest.approx(o.calNuRe()[0], rel=NU_RTOL)


def test_state_roundtrip_and_restart(oracle_mod):
    p = make("2d_rb_periodic")
    o, g = pair(oracle_mod, p)
    o.step(50)
    # load the oracle's module state into a fresh GPU lattice and continue both
    g2 = Lattice(p)
    g2.initial()
    for name in fields_for(p):
        if name in ("f_post", "g_post"):
            continue
        g2.set_state(name, o.get(FIELDS[name], field_shape(p, name)))
    o.step(50)
    g2.step(50)
    assert_same(o, g2, p, ["f", "g", "T", "u", "v"])


@pytest.mark.parametrize("precision,tol", [("fp32", 2e-3), ("fp16", 2e-2)])
def test_reduced_precision_close(oracle_mod, precision, tol):
    p = rb_params(dim=3, nx=12, ny=12, nz=12, Ra=1e5, noise_amp=1e-3, precision=precision)
    p64 = rb_params(dim=3, nx=12, ny=12, nz=12, Ra=1e5, noise_amp=1e-3)
    o = oracle_mod.Oracle(p64)
    o.initial()
    g = Lattice(p)
    g.initial()
    o.step(300)
    g.step(300)
    T = g.get_state("T")
    To = o.get(FIELDS["T"], field_shape(p64, "T"))
    assert np.abs(T - To).max() < tol
    nu_o, re_o, _ = o.calNuRe()
    nu_g, re_g = g.calNuRe()
    assert abs(nu_g - nu_o) / nu_o < 1e-2
    f = g.get_state("f")
    fo = o.get(FIELDS["f"], field_shape(p64, "f"))
    assert np.abs(f - fo).max() < tol


def test_errors_are_reported():
    p = rb_params(dim=3, n=8)
    p.nx = 2
    with pytest.raises(LbmError):
        Lattice(p)
    p = rb_params(dim=3, n=8, precision="fp32")
    g = Lattice(p)
    g.initial()
    with pytest.raises(LbmError):
        g.collision()  # stage kernels are the FP64 parity surface
    with pytest.raises(ValueError):
        g.set_state("T", np.zeros(3))


def test_divergence_detected():
    """A non-finite value planted in a host-prepared field is reported, not propagated silently."""
    p = rb_params(dim=2, nx=16, ny=8, Ra=1e5)
    g = Lattice(p)
    g.initial()
    T = g.get_state("T")
    T[3, 5] = np.nan
    g.set_state("T", T)
    g.step(3)
    with pytest.raises(LbmDiverged):
        g.calNuRe()


def test_const_division_matches_ieee(gpu_lib):
    """The plain method's 3-operation division by the reference's integer constants must
    agree bit for bit with CUDA's IEEE double division (16.7 M random normal doubles per
    constant, every 8th an exact multiple)."""
    import ctypes as C
    fn = gpu_lib.lbm_selftest_const_division
    fn.argtypes = [C.c_int64, C.c_uint64, C.POINTER(C.c_int64)]
    fn.restype = C.c_int
    for seed in (1, 20261203):
        bad = C.c_int64(-1)
        assert fn(1 << 24, seed, C.byref(bad)) == 0
        assert bad.value == 0


def test_integer_pipe_arithmetic_matches_fp64(gpu_lib):
    """Products with exact powers of two (exponent adds on the integer pipes), quotients by
    c 2^k as scaled quotients by c, and quotients through a shared correctly rounded
    reciprocal agree bit for bit with the FP64 pipe and IEEE division (2 x 16.7 M samples,
    subnormal results of the scalings included)."""
    import ctypes as C
    fn = gpu_lib.lbm_selftest_int_arith
    fn.argtypes = [C.c_int64, C.c_uint64, C.POINTER(C.c_int64)]
    fn.restype = C.c_int
    for seed in (7, 20261203):
        bad = C.c_int64(-1)
        assert fn(1 << 24, seed, C.byref(bad)) == 0
        assert bad.value == 0


@pytest.mark.parametrize("dim", [2, 3])
def test_state_transfer_direct_and_staged_agree(dim):
    """lbm_get_state / lbm_set_state through the layout kernels on the caller's host arrays
    (where the device reads pageable host memory, as a GB300 attached to Grace does) and
    through a staged copy give the same bits, both ways, for populations and scalars."""
    from lbmgpu import LBM_OPT_HOST_DIRECT, LbmError
    p = make("2d_rb_periodic" if dim == 2 else "3d_rb_noslip")
    g = Lattice(p)
    g.initial()
    g.step(30)
    names = ["f", "g", "T", "u", "rho"]
    try:
        g.set_option(LBM_OPT_HOST_DIRECT, 3)  # reads and writes
    except LbmError:
        pytest.skip("the device cannot access pageable host memory")
    direct = {k: g.get_state(k) for k in names}
    g.set_option(LBM_OPT_HOST_DIRECT, 0)
    staged = {k: g.get_state(k) for k in names}
    for k in names:
        assert np.array_equal(direct[k], staged[k]), k
    # load through one path, read back through the other
    rng = np.random.default_rng(3)
    for k in ("f", "T"):
        x = staged[k] * (1.0 + 1e-9 * rng.standard_normal(staged[k].shape))
        g.set_option(LBM_OPT_HOST_DIRECT, 1)
        g.set_state(k, x)
        g.set_option(LBM_OPT_HOST_DIRECT, 0)
        assert np.array_equal(g.get_state(k), x), k
        g.set_state(k, staged[k])
        g.set_option(LBM_OPT_HOST_DIRECT, 2)  # writes direct, reads staged
        assert np.array_equal(g.get_state(k), staged[k]), k
    g.close()
