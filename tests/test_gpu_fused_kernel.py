"""The single fused kernel (one launch per step, thermal halo in shared memory) against the
two-kernel form of the same FP32/FP16 arithmetic, and against the FP64 oracle.

Both forms evaluate the same per-cell arithmetic in FP32, and the fused kernel sums T_n
from the stored deviations in its shared-memory ring in the pull's order and form, so T and
the thermal populations agree bit for bit; the flow collision takes its macro moments from
the thermal stage instead of recomputing them, and the compiler may fuse multiply-adds
differently there, so a few flow populations differ in the last bits (measured on GB300:
up to 3e-11 in f after 6 steps in a few dozen cells).  The test allows a few units of the
storage precision.  Cases cover partial tiles (nx, ny not multiples of the 32 x 8 tile), z
chunks that do not divide nz, periodic x and z axes, and 2D.
"""
import numpy as np
import pytest

from lbmgpu import Lattice
from lbmgpu import LBM_OPT_KCHUNK, LBM_OPT_SINGLE_KERNEL
from lbmgpu.abi import FIELDS, LBM_BC_PERIODIC, LBM_BCT_PERIODIC, field_shape, rb_params

pytestmark = pytest.mark.gpu

CASES = {
    "3d_partial_tiles_kchunk3": (dict(dim=3, nx=40, ny=12, nz=8, Ra=1e6), 3, False),
    "3d_cube_kchunk16": (dict(dim=3, nx=32, ny=16, nz=20, Ra=1e6), 16, False),
    "3d_x_and_z_periodic": (dict(dim=3, nx=32, ny=10, nz=7, Ra=1e6, periodic_x=True), 4, True),
    "2d_rb_periodic": (dict(dim=2, nx=64, ny=20, Ra=1e5), 1, False),
    "2d_walls_partial": (dict(dim=2, nx=40, ny=10, Ra=1e5, periodic_x=False), 1, False),
}


# Absolute tolerances: a few units of the storage precision on the stored deviations
# (FP16 quantises a deviation of 0.02 in steps of 1.5e-5; T sums 5-7 populations).
ABS_TOL = {
    "fp32": {"T": 2e-6, "u": 5e-7, "v": 5e-7, "f": 5e-7, "g": 5e-7, "Bx_prev": 5e-7, "By_prev": 5e-7},
    "fp16": {"T": 2e-3, "u": 1e-4, "v": 1e-4, "f": 1e-4, "g": 5e-4, "Bx_prev": 1e-4, "By_prev": 1e-4},
}


def lattices(args, precision, kchunk, zper):
    out = []
    for single in (1, 0):
        p = rb_params(noise_amp=1e-3, precision=precision, **args)
        if zper:
            p.bc_flow[2] = LBM_BC_PERIODIC
            p.bc_thermal[2] = LBM_BCT_PERIODIC
        lat = Lattice(p)
        lat.set_option(LBM_OPT_SINGLE_KERNEL, single)
        lat.set_option(LBM_OPT_KCHUNK, kchunk)
        lat.initial()
        out.append(lat)
    return out


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
@pytest.mark.parametrize("case", list(CASES))
def test_single_kernel_matches_two_kernel(case, precision):
    args, kchunk, zper = CASES[case]
    a, b = lattices(args, precision, kchunk, zper)
    for chunk in (1, 40, 3):  # crosses graph capture and phase changes
        a.step(chunk)
        b.step(chunk)
        for name in ("T", "u", "v", "f", "g", "Bx_prev", "By_prev"):
            x, y = a.get_state(name), b.get_state(name)
            assert np.abs(x - y).max() <= ABS_TOL[precision][name], (name, float(np.abs(x - y).max()))
    assert a.itc == b.itc == 44
    nua, _ = a.calNuRe()
    nub, _ = b.calNuRe()
    assert nua == pytest.approx(nub, rel=1e-4 if precision == "fp32" else 5e-3)


def test_single_kernel_close_to_fp64_oracle(oracle_mod):
    p64 = rb_params(dim=3, nx=24, ny=24, nz=24, Ra=1e5, noise_amp=1e-3)
    o = oracle_mod.Oracle(p64)
    o.initial()
    o.step(400)
    p = rb_params(dim=3, nx=24, ny=24, nz=24, Ra=1e5, noise_amp=1e-3, precision="fp32")
    g = Lattice(p)
    g.set_option(LBM_OPT_KCHUNK, 5)
    g.initial()
    g.step(400)
    T = g.get_state("T")
    To = o.get(FIELDS["T"], field_shape(p64, "T"))
    assert np.abs(T - To).max() < 2e-4
    assert g.calNuRe()[0] == pytest.approx(o.calNuRe()[0], rel=1e-4)
