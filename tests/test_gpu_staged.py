"""The staged two-kernel FP32/FP16 step (tiles of x-rows brought into shared memory by
bulk asynchronous copies on an mbarrier pipeline) against the unstaged step: the same
values bit for bit, on lattices whose tiles end inside the lattice and on its faces, with
every boundary kind, in 2D and 3D; nx not a multiple of 8 falls back to the unstaged
kernels."""
import numpy as np
import pytest

from lbmgpu import LBM_OPT_PAIRS, LBM_OPT_STAGED, Lattice
from lbmgpu.abi import LBM_BC_PERIODIC, LBM_BCT_CONST, LBM_BCT_PERIODIC, LBM_CELL_SIDE, rb_params

pytestmark = pytest.mark.gpu


def cases():
    out = {
        "2d_periodic_x": rb_params(dim=2, nx=64, ny=40, Ra=1e5, noise_amp=1e-3, seed=3),
        "2d_walls_long_rows": rb_params(dim=2, nx=512, ny=24, Ra=2e5, noise_amp=1e-3, seed=4, periodic_x=False),
        "3d_noslip": rb_params(dim=3, nx=24, ny=17, nz=12, Ra=1e6, noise_amp=1e-3, seed=5),
        "3d_periodic_xz": rb_params(dim=3, nx=32, ny=10, nz=8, Ra=1e6, noise_amp=1e-3, seed=6, periodic_x=True),
        "3d_cube_40": rb_params(dim=3, n=40, Ra=1e7, noise_amp=1e-3, seed=7),
        "3d_nx_not_multiple_of_8": rb_params(dim=3, nx=20, ny=10, nz=6, Ra=1e6, noise_amp=1e-3, seed=8),
    }
    p = out["3d_periodic_xz"]
    p.bc_flow[2] = LBM_BC_PERIODIC
    p.bc_thermal[2] = LBM_BCT_PERIODIC
    side = rb_params(dim=3, nx=16, ny=10, nz=6, Ra=1e5, noise_amp=1e-3, seed=9)
    side.cell = LBM_CELL_SIDE
    side.bc_thermal[0] = LBM_BCT_CONST
    side.bc_thermal[1] = 1  # adiabatic floor and ceiling
    out["3d_side_heated"] = side
    return out


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
@pytest.mark.parametrize("name", sorted(cases()))
def test_staged_equals_unstaged(name, precision):
    p = cases()[name].copy()
    p.precision = {"fp32": 1, "fp16": 2}[precision]
    a, b = Lattice(p), Lattice(p)
    for lat, staged in ((a, 1), (b, 0)):
        lat.set_option(LBM_OPT_STAGED, staged)
        lat.set_option(LBM_OPT_PAIRS, 0)
        lat.initial()
        lat.step(70)  # first step, single steps and two graph chunks
    a.sync()
    for field in ("f", "g", "T", "u", "v", "Bx_prev", "By_prev"):
        x, y = a.get_state(field), b.get_state(field)
        assert np.array_equal(x, y), (name, precision, field, float(np.abs(x - y).max()))
