"""GPU tests of the fixed arithmetic of FP64 handles (lbm_params.arith = LBM_ARITH_FIXED).

* The kernels equal the host stepper of the same cell bodies bit for bit (integer
  arithmetic), across a captured graph chunk, on five switch sets.
* On the 128^3 Rayleigh-Benard cube at Ra 1e7 (the benchmark workload), 1000 fused steps
  stay within 1e-12 of the plain method in every population (which equals the oracle bit
  for bit) and within 1e-10 in Nu and Re.
* Reading diagnostics does not change the run; stage kernels and state loads after fixed
  steps continue within the same tolerance.
"""
import numpy as np
import pytest

from lbmgpu import Lattice
from lbmgpu.abi import FIELDS, field_shape, rb_params

from test_cpu_fixed import build_stepper, cases, run_fixed, state_arrays

pytestmark = pytest.mark.gpu

POP_RTOL = 1e-12   # populations after 1000 steps
NU_RTOL = 1e-10    # Nusselt / Reynolds numbers


@pytest.fixture(scope="module")
def stepper(tmp_path_factory):
    return build_stepper(tmp_path_factory.mktemp("fixedgpu"))


def fixed(p):
    q = p.copy()
    q.arith = 1
    return q


def module_fields(p):
    names = ["f", "g", "rho", "u", "v", "T", "Bx_prev", "By_prev"]
    return names + (["w", "Bz_prev"] if p.dim == 3 else ["Fx", "Fy"])


@pytest.mark.parametrize("name", sorted(cases()))
def test_fixed_kernels_equal_host_stepper(gpu_lib, oracle_mod, stepper, name):
    from lbmgpu.abi import LbmConstants
    p = fixed(cases()[name])
    steps = 40  # the first step, a captured chunk of 32 steps, single steps
    o = oracle_mod.Oracle(cases()[name])
    o.initial()
    c = o.constants(LbmConstants)
    st = run_fixed(stepper, p, c, state_arrays(o, cases()[name]), steps)
    o.close()
    g = Lattice(p)
    g.initial()
    g.step(steps)
    for k in module_fields(p):
        a = g.get_state(k)
        key = k
        assert np.array_equal(a, st[key]), "%s: %s differs (max |d| %g)" % (name, k, np.abs(a - st[key]).max())
    g.close()


def test_fixed_vs_plain_128cube_1000_steps(gpu_lib):
    """The benchmark workload: 128^3, Ra 1e7, Pr 0.71, U 0.1, seeded noise."""
    base = rb_params(dim=3, n=128, Ra=1e7, Pr=0.71, U=0.1, noise_amp=1e-3, seed=20261203)
    a = Lattice(base)
    b = Lattice(fixed(base))
    for lat in (a, b):
        lat.initial()
        lat.step(1000)
    fa, fb = a.get_state("f"), b.get_state("f")
    assert float(np.max(np.abs(fb - fa) / np.abs(fa))) <= POP_RTOL
    ga, gb = a.get_state("g"), b.get_state("g")
    assert float(np.max(np.abs(gb - ga)) / np.max(np.abs(ga))) <= POP_RTOL
    nua, rea = a.calNuRe()
    nub, reb = b.calNuRe()
    assert abs(nub - nua) <= NU_RTOL * abs(nua)
    assert abs(reb - rea) <= NU_RTOL * abs(rea)
    a.close()
    b.close()


def test_fixed_diagnostics_do_not_change_the_run(gpu_lib):
    p = fixed(rb_params(dim=3, n=20, Ra=1e6, noise_amp=1e-3))
    a, b = Lattice(p), Lattice(p)
    a.initial()
    b.initial()
    for _ in range(8):
        a.step(8)
        a.calNuRe()
        a.get_state("T")
    b.step(64)
    for k in ("f", "g", "T", "u"):
        assert np.array_equal(a.get_state(k), b.get_state(k)), k
    a.close()
    b.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_fixed_stage_kernels_and_loads_continue(gpu_lib, dim):
    """After fixed steps, the stage entry points (which run the plain method's kernels on
    the FP64 module arrays) and a state load continue from the fixed state; the result stays
    within the tolerance of the plain method doing the same."""
    base = rb_params(dim=2, nx=32, ny=16, Ra=1e5, noise_amp=1e-3) if dim == 2 else \
        rb_params(dim=3, n=12, Ra=1e6, noise_amp=1e-3)
    a, b = Lattice(base), Lattice(fixed(base))
    for lat in (a, b):
        lat.initial()
        lat.step(10)
        lat.stage_step()
        lat.step(5)
        f = lat.get_state("f")
        lat.set_state("f", f)
        lat.step(40)
    for k in ("f", "g", "T"):
        x, y = a.get_state(k), b.get_state(k)
        assert float(np.max(np.abs(y - x)) / np.max(np.abs(x))) <= POP_RTOL, k
    assert abs(a.calNuRe()[0] - b.calNuRe()[0]) <= NU_RTOL * abs(a.calNuRe()[0])
    a.close()
    b.close()


def test_fixed_kernel_timing_hook(gpu_lib):
    p = fixed(rb_params(dim=3, n=24, Ra=1e6, noise_amp=1e-3))
    lat = Lattice(p)
    lat.initial()
    tf, tt = lat.time_kernels(4)  # fused passes: the whole step in the first figure
    assert tf > 0.0 and tt >= 0.0
    lat.close()


@pytest.mark.parametrize("shape,periodic", [((64, 48, 40), False), ((48, 40, 36), True), ((300, 20, 34), False),
                                            ((100, 17, 50), True)])
def test_fixed_fused_pass_equals_two_kernel_step(gpu_lib, shape, periodic):
    """The fused pass (thermal of step s and flow of step s+1 in one launch, T summed from
    pushed values in shared memory) against the two-kernel step, bit for bit: several row
    tiles and z chunks, block widths 64..384, walls and x/z-periodic faces."""
    from lbmgpu import LBM_OPT_SINGLE_KERNEL
    nx, ny, nz = shape
    p = rb_params(dim=3, nx=nx, ny=ny, nz=nz, Ra=1e6, noise_amp=1e-3, precision="fp64x", periodic_x=periodic,
                  legacy_thermal=periodic)
    if periodic:
        p.bc_flow[2] = 1
        p.bc_thermal[2] = 2
    a, b = Lattice(p), Lattice(p)
    a.set_option(LBM_OPT_SINGLE_KERNEL, 0)
    b.set_option(LBM_OPT_SINGLE_KERNEL, 1)
    for lat in (a, b):
        lat.initial()
        lat.step(70)   # first step, enter, a captured chunk of 32 passes, single passes, exit
        lat.step(5)
    for k in ("f", "g", "T", "u", "w", "Bx_prev", "Bz_prev"):
        assert np.array_equal(a.get_state(k), b.get_state(k)), k
    a.close()
    b.close()


@pytest.mark.parametrize("name", ["rb2d_periodic", "rb3d_noslip", "rb3d_periodic_legacy"])
def test_wide_and_narrow_indices_agree(gpu_lib, name):
    """The interior-row kernels with 32-bit cell indices (the default where every index
    fits) and with 64-bit ones (the form of lattices with q * ncell >= 2^31) give the same
    bits, across a captured chunk and single steps."""
    from lbmgpu import LBM_OPT_WIDE_INDEX
    p = fixed(cases()[name])
    a, b = Lattice(p), Lattice(p)
    b.set_option(LBM_OPT_WIDE_INDEX, 1)
    for lat in (a, b):
        lat.initial()
        lat.step(45)
    for k in module_fields(p):
        assert np.array_equal(a.get_state(k), b.get_state(k)), k
    a.close()
    b.close()
