"""The paired two-kernel FP32/FP16 step (two x-adjacent cells per thread, 2-cell vector
loads and stores) and the row form (interior rows with select-based x pulls, face rows with
the full boundary rule) against the one-cell-per-thread step: the same values, bit for bit,
on lattices with every boundary kind on the x faces (the faces where a pair is split into a
vector part and a scalar boundary part), and the fallback for odd nx."""
import numpy as np
import pytest

from lbmgpu import LBM_OPT_PAIRS, LBM_OPT_ROWS, Lattice
from lbmgpu.abi import LBM_BC_PERIODIC, LBM_BCT_CONST, LBM_BCT_PERIODIC, LBM_CELL_SIDE, rb_params

pytestmark = pytest.mark.gpu


def cases():
    out = {
        "2d_periodic_x": rb_params(dim=2, nx=64, ny=32, Ra=1e5, noise_amp=1e-3, seed=3),
        "2d_walls": rb_params(dim=2, nx=48, ny=24, Ra=2e5, noise_amp=1e-3, seed=4, periodic_x=False),
        "3d_noslip": rb_params(dim=3, nx=20, ny=16, nz=12, Ra=1e6, noise_amp=1e-3, seed=5),
        "3d_periodic_xz": rb_params(dim=3, nx=24, ny=10, nz=8, Ra=1e6, noise_amp=1e-3, seed=6, periodic_x=True),
        "3d_odd_nx": rb_params(dim=3, nx=15, ny=10, nz=6, Ra=1e6, noise_amp=1e-3, seed=7),
        "3d_wide_row": rb_params(dim=3, nx=160, ny=6, nz=5, Ra=1e6, noise_amp=1e-3, seed=8),
    }
    p = out["3d_periodic_xz"]
    p.bc_flow[2] = LBM_BC_PERIODIC
    p.bc_thermal[2] = LBM_BCT_PERIODIC
    side = rb_params(dim=3, nx=12, ny=10, nz=6, Ra=1e5, noise_amp=1e-3, seed=9)
    side.cell = LBM_CELL_SIDE
    side.bc_thermal[0] = LBM_BCT_CONST
    side.bc_thermal[1] = 1  # adiabatic floor and ceiling
    out["3d_side_heated"] = side
    return out


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
@pytest.mark.parametrize("name", sorted(cases()))
def test_paired_equals_one_cell(name, precision):
    p = cases()[name].copy()
    p.precision = {"fp32": 1, "fp16": 2}[precision]
    a, b = Lattice(p), Lattice(p)
    a.set_option(LBM_OPT_PAIRS, 1)
    b.set_option(LBM_OPT_PAIRS, 0)
    for lat in (a, b):
        lat.initial()
        lat.step(70)  # first step, single steps and two graph chunks
    for field in ("f", "g", "T", "u", "v", "Bx_prev", "By_prev"):
        x, y = a.get_state(field), b.get_state(field)
        assert np.array_equal(x, y), (name, precision, field, float(np.abs(x - y).max()))


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
@pytest.mark.parametrize("name", sorted(cases()))
def test_rows_equal_one_cell(name, precision):
    p = cases()[name].copy()
    p.precision = {"fp32": 1, "fp16": 2}[precision]
    a, b = Lattice(p), Lattice(p)
    for lat, rows in ((a, 1), (b, 0)):
        lat.set_option(LBM_OPT_PAIRS, 0)
        lat.set_option(LBM_OPT_ROWS, rows)
        lat.initial()
        lat.step(70)  # first step, single steps and two graph chunks
    for field in ("f", "g", "T", "u", "v", "Bx_prev", "By_prev"):
        x, y = a.get_state(field), b.get_state(field)
        assert np.array_equal(x, y), (name, precision, field, float(np.abs(x - y).max()))
    a.close()
    b.close()


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
@pytest.mark.parametrize("name", sorted(cases()))
def test_wide_index_equals_narrow(name, precision):
    """The one-cell kernels with 32-bit cell indices (the default where every index fits) and
    with 64-bit ones give the same bits."""
    from lbmgpu import LBM_OPT_WIDE_INDEX
    p = cases()[name].copy()
    p.precision = {"fp32": 1, "fp16": 2}[precision]
    a, b = Lattice(p), Lattice(p)
    for lat, wide in ((a, 0), (b, 1)):
        lat.set_option(LBM_OPT_PAIRS, 0)
        lat.set_option(LBM_OPT_WIDE_INDEX, wide)
        lat.initial()
        lat.step(70)
    for field in ("f", "g", "T", "u", "v", "Bx_prev", "By_prev"):
        x, y = a.get_state(field), b.get_state(field)
        assert np.array_equal(x, y), (name, precision, field, float(np.abs(x - y).max()))
    a.close()
    b.close()
