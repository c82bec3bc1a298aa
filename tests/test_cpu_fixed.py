"""The fixed arithmetic of FP64 handles (csrc/lbm_fixed_cell.cuh) against the oracle, on the CPU.

The GPU kernels' cell bodies run through a host stepper (fixed_cell_check.cpp) from the
oracle's initial state; after 1000 steps the populations and the oracle's own Nu/Re of the
resulting state are compared with the oracle's run:

* populations f within 1e-12 relative (element by element), g within 1e-12 of max|g|,
  Nu and Re within 1e-10 relative (the plain method's tolerance for a non-bitwise FP64 path);
* where the flow itself amplifies rounding (3D no-slip, Ra 1e6 on 10 x 9 x 8 cells: the
  convective instability grows through these steps), the bar is the distance between the
  oracle and the same oracle compiled with FMA contraction -- what gfortran -O2 produces
  for the reference on aarch64 -- times 10.

Also: conservation of mass to the last bit of the integer format, the rejection of
parameters the form does not take, and the range check of its constants."""
import ctypes as C
import os
import platform
import shutil
import subprocess

import numpy as np
import pytest

from lbmgpu.abi import (FIELDS, LBM_ARITH_FIXED, LBM_BCT_ADIABATIC, LBM_BCT_CONST, LBM_CELL_SIDE, LbmConstants,
                        field_shape, rb_params)

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DP = C.POINTER(C.c_double)
STEPS = 1000


def _cxx():
    cxx = shutil.which("g++") or shutil.which("c++")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if not cxx or not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("no C++ compiler or CUDA headers")
    return cxx, cuda_inc


def build_stepper(outdir):
    """Compile the host stepper of the fixed arithmetic; returns the loaded library."""
    cxx, cuda_inc = _cxx()
    so = os.path.join(str(outdir), "libfixedcell.so")
    cmd = [cxx, "-std=c++17", "-O2", "-shared", "-fPIC", "-I", os.path.join(ROOT, "-2d-3d-_gb300", "csrc"), "-I",
           os.path.join(ROOT, "include"), "-I", cuda_inc, "-o", so, os.path.join(HERE, "fixed_cell_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(so)
    lib.fixed_run.restype = C.c_int
    lib.fixed_constants_ok.restype = C.c_int
    return lib


@pytest.fixture(scope="module")
def stepper(tmp_path_factory):
    return build_stepper(tmp_path_factory.mktemp("fixed"))


def cases():
    side = rb_params(dim=3, nx=10, ny=8, nz=6, Ra=1e5, noise_amp=1e-3, seed=8)
    side.cell = LBM_CELL_SIDE
    side.bc_thermal[0] = LBM_BCT_CONST
    side.bc_thermal[1] = LBM_BCT_ADIABATIC
    legacy = rb_params(dim=3, nx=9, ny=8, nz=7, Ra=1e5, U=0.02, noise_amp=1e-3, seed=6, periodic_x=True,
                       legacy_thermal=True)
    legacy.bc_flow[2] = 1
    legacy.bc_thermal[2] = 2
    return {
        "rb2d_periodic": rb_params(dim=2, nx=24, ny=12, Ra=1e5, noise_amp=1e-3, seed=3),
        "rb2d_walls_nog": rb_params(dim=2, nx=20, ny=14, Ra=2e5, noise_amp=1e-3, seed=4, periodic_x=False,
                                    use_g=False),
        "rb3d_noslip": rb_params(dim=3, nx=10, ny=9, nz=8, Ra=1e6, noise_amp=1e-3, seed=5),
        "rb3d_periodic_legacy": legacy,
        "side3d": side,
        # two planes in z: no interior rows, the face-row kernels hold every cell
        "rb3d_two_planes": rb_params(dim=3, nx=12, ny=8, nz=2, Ra=1e5, noise_amp=1e-3, seed=9),
    }


# cases whose flow amplifies rounding over the compared steps (see the module docstring)
AMPLIFYING = {"rb3d_noslip"}


def state_arrays(o, p):
    """The module state the stepper takes, from an oracle, in the Fortran layout."""
    d3 = p.dim == 3
    out = {}
    for k in ("f", "g", "rho", "u", "v", "w", "T", "Bx_prev", "By_prev", "Bz_prev", "Fx", "Fy"):
        if (k in ("w", "Bz_prev") and not d3) or (k in ("Fx", "Fy") and d3):
            out[k] = None
        else:
            out[k] = np.ascontiguousarray(o.get(FIELDS[k], field_shape(p, k)))
    return out


def run_fixed(lib, p, c, st, steps):
    def ptr(a):
        return a.ctypes.data_as(DP) if a is not None else None
    tl = np.zeros(field_shape(p, "T")) if p.dim == 3 else None
    rc = lib.fixed_run(C.byref(p), C.byref(c), C.c_longlong(steps), ptr(st["f"]), ptr(st["g"]), ptr(st["rho"]),
                       ptr(st["u"]), ptr(st["v"]), ptr(st["w"]), ptr(st["T"]), ptr(st["Bx_prev"]),
                       ptr(st["By_prev"]), ptr(st["Bz_prev"]), ptr(st["Fx"]), ptr(st["Fy"]), ptr(tl))
    assert rc == 0
    return st


def distances(p, st, o):
    """(f elementwise relative, g relative to max|g|) between a state and an oracle."""
    f = o.get(FIELDS["f"], field_shape(p, "f"))
    g = o.get(FIELDS["g"], field_shape(p, "g"))
    return (float(np.max(np.abs(st["f"] - f) / np.abs(f))), float(np.max(np.abs(st["g"] - g)) / np.max(np.abs(g))))


def nu_re_of_state(oracle_mod, p, st):
    """The oracle's calNuRe of a given module state."""
    o = oracle_mod.Oracle(p)
    o.initial()
    for k in ("f", "g", "rho", "u", "v", "w", "T"):
        if st.get(k) is not None:
            o.set(FIELDS[k], st[k])
    nu, re, _ = o.calNuRe()
    o.close()
    return nu, re


def fma_oracle(outdir, oracle_mod):
    """The oracle compiled with FMA contraction (the reference as gfortran -O2 builds it on
    aarch64), loaded as a separate module; None when no FMA code generation is available."""
    cxx, _ = _cxx()
    flags = ["-ffp-contract=fast"]
    if platform.machine() in ("x86_64", "AMD64"):
        try:
            with open("/proc/cpuinfo") as fh:
                if " fma" not in fh.read():
                    return None
        except OSError:
            return None
        flags.append("-mfma")
    so = os.path.join(str(outdir), "liboracle_fma.so")
    src = os.path.join(ROOT, "oracle", "lbm_oracle.cpp")
    r = subprocess.run([cxx, "-std=c++17", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", so, src] + flags,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    import importlib.util
    spec = importlib.util.spec_from_file_location("oracle_fma", oracle_mod.__file__)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build = lambda *a, **k: so
    return mod


@pytest.mark.parametrize("name", sorted(cases()))
def test_fixed_matches_oracle_after_1000_steps(stepper, oracle_mod, tmp_path, name):
    p = cases()[name]
    o = oracle_mod.Oracle(p)
    o.initial()
    c = o.constants(LbmConstants)
    st = run_fixed(stepper, p, c, state_arrays(o, p), STEPS)
    o.step(STEPS)
    df, dg = distances(p, st, o)
    nu_o, re_o, _ = o.calNuRe()
    nu_x, re_x = nu_re_of_state(oracle_mod, p, st)
    bar_f = bar_g = 1e-12
    bar_nu = 1e-10
    if name in AMPLIFYING:
        fm = fma_oracle(tmp_path, oracle_mod)
        if fm is None:
            pytest.skip("no FMA code generation on this host to calibrate the amplifying case")
        of = fm.Oracle(p)
        of.initial()
        of.step(STEPS)
        ff, fg = distances(p, state_arrays(of, p), o)
        nu_f, re_f, _ = of.calNuRe()
        of.close()
        bar_f, bar_g = max(bar_f, 10 * ff), max(bar_g, 10 * fg)
        bar_nu = max(bar_nu, 10 * abs(nu_f - nu_o) / abs(nu_o))
    assert df <= bar_f, (name, df, bar_f)
    assert dg <= bar_g, (name, dg, bar_g)
    assert abs(nu_x - nu_o) <= bar_nu * abs(nu_o), (name, nu_x, nu_o)
    assert abs(re_x - re_o) <= 1e-10 * abs(re_o) or name in AMPLIFYING, (name, re_x, re_o)
    o.close()


@pytest.mark.parametrize("name", ["rb2d_walls_nog", "rb3d_noslip"])
def test_fixed_conserves_mass_exactly(stepper, oracle_mod, name):
    """Half-way bounce-back moves populations without loss and the collision's update has
    zero sum (every moment row but the first sums to zero), so on a lattice closed by walls
    the total mass of the integer state never changes.  Checked on the materialised
    rho = 1 + sum d, each rounded once to FP64.  (An x-periodic face does not conserve mass
    in the reference: its diagonal directions are copied from the same row, 2DRB.F90:821-828;
    the fixed form reproduces that loss.)"""
    p = cases()[name]
    o = oracle_mod.Oracle(p)
    o.initial()
    c = o.constants(LbmConstants)
    s0 = state_arrays(o, p)
    s1 = run_fixed(stepper, p, c, state_arrays(o, p), 1)
    s2 = run_fixed(stepper, p, c, state_arrays(o, p), 300)
    m1 = np.sum(np.round((s1["rho"] - 1.0) * 2.0 ** 60))
    m2 = np.sum(np.round((s2["rho"] - 1.0) * 2.0 ** 60))
    # the materialised rho is rounded once to FP64: bound the sum by that rounding only
    tol = s0["rho"].size * 2.0 ** 60 * 2.0 ** -53
    assert abs(m2 - m1) <= tol
    o.close()


def test_fixed_parameters(stepper, oracle_mod):
    import lbmgpu
    p = rb_params(dim=3, n=12, Ra=1e6, precision="fp64x")
    assert p.arith == LBM_ARITH_FIXED and p.precision == 0
    assert lbmgpu.footprint(p) > lbmgpu.footprint(rb_params(dim=3, n=12, Ra=1e6))
    for bad in ("AA", "ha", "fp32"):
        q = rb_params(dim=2, ny=16, Ra=1e5, precision="fp64x")
        if bad == "AA":
            q.pattern = 1
        elif bad == "ha":
            q.side_heated_ha = 1
        else:
            q.precision = 1
        with pytest.raises(lbmgpu.LbmError):
            lbmgpu.footprint(q)
    o = oracle_mod.Oracle(p)
    c = o.constants(LbmConstants)
    assert stepper.fixed_constants_ok(C.byref(p), C.byref(c)) == 0
    o.close()


def test_fixed_stepper_is_clean_under_sanitizers(tmp_path):
    """The shared cell code (pull with boundary rules, the fixed-arithmetic bodies) built for
    the CPU with -DLBM_CHECK (index asserts on every computed source cell) and the address and
    undefined-behaviour sanitizers, run over every switch set: no out-of-range access, no
    assert, no undefined operation.  This stands in for a device-side bounds check."""
    import sys
    cxx, cuda_inc = _cxx()
    asan = subprocess.run([cxx, "-print-file-name=libasan.so"], capture_output=True, text=True).stdout.strip()
    if not asan or not os.path.isabs(asan) or not os.path.exists(asan):
        pytest.skip("no AddressSanitizer runtime")
    so = str(tmp_path / "libfixed_san.so")
    cmd = [cxx, "-std=c++17", "-O1", "-g", "-DLBM_CHECK", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=undefined", "-shared", "-fPIC", "-I", os.path.join(ROOT, "-2d-3d-_gb300", "csrc"),
           "-I", os.path.join(ROOT, "include"), "-I", cuda_inc, "-o", so, os.path.join(HERE, "fixed_cell_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    script = (
        "import sys, ctypes as C\n"
        "sys.path[:0] = [%r, %r, %r]\n"
        "import test_cpu_fixed as T\n"
        "from lbmgpu.abi import LbmConstants\n"
        "from oracle import oracle as ora\n"
        "lib = C.CDLL(%r); lib.fixed_run.restype = C.c_int\n"
        "for name, p in T.cases().items():\n"
        "    o = ora.Oracle(p); o.initial(); c = o.constants(LbmConstants)\n"
        "    T.run_fixed(lib, p, c, T.state_arrays(o, p), 12)\n"
        "    o.close()\n"
        "print('clean')\n" % (ROOT, os.path.join(ROOT, "-2d-3d-_gb300"), HERE, so))
    env = dict(os.environ, LD_PRELOAD=asan, ASAN_OPTIONS="detect_leaks=0")
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0 and "clean" in r.stdout, r.stdout[-2000:] + r.stderr[-4000:]
