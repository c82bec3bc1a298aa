"""The plain method's per-cell FP64 arithmetic against the oracle's stages, on the CPU.

The GPU kernels' collision, macro and thermal-collision functions (csrc/lbm_exact_cell.cuh)
are compiled for the host (exact_cell_check.cpp) and applied to every cell of a stepped
lattice; their outputs must equal the oracle's collision, macro and collisionT stages bit
for bit.  This covers the routes the kernels take to the reference's bits without the
reference's instruction sequence:

* products with exact powers of two as exponent adds;
* rate-only factors rounded once on the host;
* a quotient by c*2^k as the scaled quotient by c;
* the macro step's quotients through one correctly rounded reciprocal;
* conserved moments without the zero-rate terms;
* the fused kernels' forms that take m0 and the momentum sums (flow) or n0 (thermal) from
  the other kernel.

Six switch sets are covered: 2D RB with x periodic and with walls, M1G off; 2D side-heated
with the magnetic force; 3D RB no-slip; 3D x/z-periodic with the legacy thermal scheme;
3D side-heated."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from lbmgpu.abi import (FIELDS, LBM_BC_PERIODIC, LBM_BCT_ADIABATIC, LBM_BCT_CONST, LBM_BCT_PERIODIC, LBM_CELL_SIDE,
                        LbmConstants, field_shape, rb_params)

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DP = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def cells(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("no CUDA headers")
    so = str(tmp_path_factory.mktemp("cell") / "libexactcell.so")
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-I",
           os.path.join(ROOT, "-2d-3d-_gb300", "csrc"), "-I", os.path.join(ROOT, "include"), "-I", cuda_inc, "-o", so,
           os.path.join(HERE, "exact_cell_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return C.CDLL(so)


def cases():
    out = {
        "rb2d_periodic": rb_params(dim=2, nx=24, ny=12, Ra=1e5, noise_amp=1e-3, seed=3),
        "rb2d_walls_nog": rb_params(dim=2, nx=20, ny=14, Ra=2e5, noise_amp=1e-3, seed=4, periodic_x=False),
        "rb3d_noslip": rb_params(dim=3, nx=10, ny=9, nz=8, Ra=1e6, noise_amp=1e-3, seed=5),
        "rb3d_periodic_legacy": rb_params(dim=3, nx=9, ny=8, nz=7, Ra=1e5, U=0.02, noise_amp=1e-3, seed=6,
                                          periodic_x=True, legacy_thermal=True),
    }
    out["rb2d_walls_nog"].use_g = 0
    p = out["rb3d_periodic_legacy"]
    p.bc_flow[2] = LBM_BC_PERIODIC
    p.bc_thermal[2] = LBM_BCT_PERIODIC
    for dim, name in ((2, "side2d_ha"), (3, "side3d")):
        s = rb_params(dim=dim, nx=16, ny=16, nz=6, Ra=1e5, noise_amp=1e-3, seed=7, periodic_x=False) if dim == 2 else \
            rb_params(dim=3, nx=10, ny=8, nz=6, Ra=1e5, noise_amp=1e-3, seed=8)
        s.cell = LBM_CELL_SIDE
        s.bc_thermal[0] = LBM_BCT_CONST
        s.bc_thermal[1] = LBM_BCT_ADIABATIC
        if dim == 2:
            s.side_heated_ha, s.Ha, s.phi_deg = 1, 15.0, 30.0
        out[name] = s
    return out


def ptr(a):
    return a.ctypes.data_as(DP)


def arr(o, p, name):
    return np.ascontiguousarray(o.get(FIELDS[name], field_shape(p, name)), dtype=np.float64).ravel()


@pytest.mark.parametrize("name", sorted(cases()))
def test_cell_arithmetic_equals_oracle_stages(cells, oracle_mod, name):
    p = cases()[name]
    d3 = p.dim == 3
    n = p.nx * p.ny * (p.nz if d3 else 1)
    o = oracle_mod.Oracle(p)
    o.initial()
    o.step(3)
    c = o.constants(LbmConstants)
    zero = np.zeros(n)

    # collision from the module state (both forms)
    f, rho, u, v, T = (arr(o, p, k) for k in ("f", "rho", "u", "v", "T"))
    w = arr(o, p, "w") if d3 else zero
    o.collision()
    want = arr(o, p, "f_post")
    for known in (0, 1):
        fp, fx, fy = np.empty_like(f), np.empty(n), np.empty(n)
        cells.cell_collide(p.dim, C.byref(p), C.byref(c), C.c_longlong(n), ptr(f), ptr(rho), ptr(u), ptr(v), ptr(w),
                           ptr(T), known, ptr(fp), ptr(fx), ptr(fy))
        assert np.array_equal(fp, want), (name, "collision", known)
        if not d3:
            assert np.array_equal(fx, arr(o, p, "Fx")) and np.array_equal(fy, arr(o, p, "Fy")), (name, known)

    # macro of the streamed populations
    o.streaming()
    o.bounceback()
    f = arr(o, p, "f")
    lag0, lag1 = (arr(o, p, "Fx"), arr(o, p, "Fy")) if not d3 else (arr(o, p, "T"), zero)
    o.macro()
    out = [np.empty(n) for _ in range(4)]
    cells.cell_macro(p.dim, C.byref(p), C.byref(c), C.c_longlong(n), ptr(f), ptr(lag0), ptr(lag1), *[ptr(a) for a in out])
    for k, got in zip(("rho", "u", "v", "w"), out):
        if k == "w" and not d3:
            continue
        assert np.array_equal(got, arr(o, p, k)), (name, "macro", k)

    # thermal collision (both forms)
    g, u, v, T = (arr(o, p, k) for k in ("g", "u", "v", "T"))
    w = arr(o, p, "w") if d3 else zero
    bx, by = arr(o, p, "Bx_prev"), arr(o, p, "By_prev")
    bz = arr(o, p, "Bz_prev") if d3 else zero
    o.collisionT()
    want = arr(o, p, "g_post")
    bnew = [arr(o, p, "Bx_prev"), arr(o, p, "By_prev")] + ([arr(o, p, "Bz_prev")] if d3 else [])
    for known in (0, 1):
        gp, b0, b1, b2 = np.empty_like(g), np.empty(n), np.empty(n), np.empty(n)
        cells.cell_collideT(p.dim, C.byref(p), C.byref(c), C.c_longlong(n), ptr(g), ptr(u), ptr(v), ptr(w), ptr(T),
                            ptr(bx), ptr(by), ptr(bz), known, ptr(gp), ptr(b0), ptr(b1), ptr(b2))
        assert np.array_equal(gp, want), (name, "collisionT", known)
        if p.use_g:
            for got, ref in zip((b0, b1, b2), bnew):
                assert np.array_equal(got, ref), (name, "B", known)
    o.close()
