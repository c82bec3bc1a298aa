"""The allocation-free Nu/Re entry point, checked against the regular one.

lbm_calNuRe_noalloc exists for callers that cannot let a library call cudaMalloc: their
device memory is owned by an allocator of their own (the Fortran driver's OpenACC data
region or pool, a framework's caching allocator, a server with a fixed HBM budget), where
a library allocation can fail or escape the owner's accounting and cudaFree synchronises
the device.  This test calls it through the C ABI on fields the test itself places on
the GPU, twice in a row (the shared scratch array keeps the previous call's contents),
and compares with lbm_calNuRe of the same state within the tolerance the parity tests use.
It lives in its own file, collected last, and passes alone or after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NU_RTOL = 1e-10
LBM_ERR_TOO_LARGE = 7
LBM_NOALLOC_MAX_CELLS = 1216 * 65536


def _bind(lib):
    fn = lib.lbm_calNuRe_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_double, C.c_double,
                   C.c_double, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    fn.restype = C.c_int
    return fn


def _lattice(case):
    from lbmgpu.abi import LBM_BCT_ADIABATIC, LBM_BCT_CONST, LBM_CELL_SIDE, rb_params
    if case == "3d_128":  # a multi-block lattice: every block strides over many cells
        return rb_params(dim=3, n=128, Ra=1e7, noise_amp=1e-3), 0
    if case == "2d_20":
        return rb_params(dim=2, ny=20, Ra=1e6, noise_amp=1e-3), 0
    p = rb_params(dim=3, nx=24, ny=20, nz=12, Ra=1e5, noise_amp=1e-3, seed=8)  # side-heated: Nu from <u T>
    p.cell = LBM_CELL_SIDE
    p.bc_thermal[0] = LBM_BCT_CONST
    p.bc_thermal[1] = LBM_BCT_ADIABATIC
    return p, 1


@pytest.mark.parametrize("case", ["3d_128", "2d_20", "3d_side"])
def test_noalloc_nu_re_matches_calNuRe(gpu_lib, case):
    import torch
    from lbmgpu import Lattice
    fn = _bind(gpu_lib)
    p, side = _lattice(case)
    dim = p.dim
    lat = Lattice(p)
    lat.initial()
    lat.step(150)
    nu_ref, re_ref = lat.calNuRe()
    c = lat.constants()
    names = ["u", "v", "T"] + (["w"] if dim == 3 else [])
    dev = {k: torch.tensor(np.ascontiguousarray(lat.get_state(k)), dtype=torch.float64, device="cuda") for k in names}
    torch.cuda.synchronize()
    ncell = dev["T"].numel()
    wptr = dev["w"].data_ptr() if dim == 3 else None
    for _ in range(2):
        nu, re = C.c_double(), C.c_double()
        st = fn(dev["u"].data_ptr(), dev["v"].data_ptr(), wptr, dev["T"].data_ptr(), ncell, side,
                c["lengthUnit"], c["diffusivity"], c["viscosity"], None, C.byref(nu), C.byref(re))
        assert st == 0
        assert nu.value == pytest.approx(nu_ref, rel=NU_RTOL)
        assert re.value == pytest.approx(re_ref, rel=NU_RTOL)
    # a lattice beyond the fixed scratch capacity is rejected before anything is launched
    nu, re = C.c_double(), C.c_double()
    st = fn(dev["u"].data_ptr(), dev["v"].data_ptr(), wptr, dev["T"].data_ptr(), LBM_NOALLOC_MAX_CELLS + 1, side,
            c["lengthUnit"], c["diffusivity"], c["viscosity"], None, C.byref(nu), C.byref(re))
    assert st == LBM_ERR_TOO_LARGE
    lat.close()
