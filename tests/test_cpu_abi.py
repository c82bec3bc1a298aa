"""C-ABI checks that need no GPU: the library loads, exports every symbol the headers
declare, fills the parameter struct consistently with the Python mirror, and derives the
same constants as the oracle (host-only calls; no kernel is launched)."""
import ctypes as C
import glob
import os
import re

import pytest

from lbmgpu.abi import LbmConstants, LbmParams, rb_params

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s+\**\s*(lbm_[A-Za-z0-9_]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_header_declares_the_reference_surface():
    names = declared_functions()
    for sub in ("collision", "streaming", "bounceback", "macro", "collisionT", "streamingT", "bouncebackT",
                "macroT", "initial", "check", "calNuRe", "RBcalc_Nu_global", "RBcalc_Nu_wall_avg",
                "SideHeatedcalc_Nu_global", "SideHeatedcalc_Nu_wall_avg", "SideHeatedcalc_umid_max",
                "SideHeatedcalc_vmid_max", "SideHeatedcalc_wmid_max", "RBcalc_umid_max", "RBcalc_vmid_max",
                "RBcalc_wmid_max", "backupData", "reload"):
        assert "lbm_" + sub in names


def test_python_signatures_cover_the_header():
    import lbmgpu
    missing = [n for n in sorted(declared_functions()) if n not in lbmgpu.SIGNATURES]
    # entry points bound elsewhere (tests call them through ctypes directly)
    assert set(missing) <= {"lbm_selftest_const_division", "lbm_selftest_int_arith", "lbm_calNuRe_noalloc"}, missing


def test_library_exports_every_declared_symbol(gpu_lib):
    missing = [n for n in sorted(declared_functions()) if not hasattr(gpu_lib, n)]
    assert not missing, missing


def test_params_struct_layout(gpu_lib):
    import lbmgpu
    p = lbmgpu.params_default(2)
    assert (p.dim, p.nx, p.ny, p.nz) == (2, 320, 160, 1)
    assert p.Ra == 5e4 and p.Pr == 0.71 and p.Mach == 0.1 and p.Thot == 0.5 and p.Tcold == -0.5
    assert list(p.bc_flow) == [1, 0, 0] and list(p.bc_thermal) == [2, 0, 1]
    assert p.use_g == 1 and p.legacy_thermal == 0 and p.seed == 20261203 and p.noise_amp == 0.0
    p3 = lbmgpu.params_default(3)
    assert (p3.nx, p3.ny, p3.nz, p3.Ra) == (120, 120, 120, 1e7)
    assert C.sizeof(LbmParams) == 144
    assert (p.side_heated_ha, p.Ha, p.phi_deg) == (0, 20.0, 0.0)


@pytest.mark.parametrize("dim,legacy", [(2, False), (3, False), (2, True), (3, True)])
def test_constants_equal_oracle(gpu_lib, oracle_mod, dim, legacy):
    import lbmgpu
    p = rb_params(dim=dim, n=64, ny=64, Ra=1e6, U=0.02 if legacy else 0.1, legacy_thermal=legacy)
    c_lib = lbmgpu.derive_constants(p).as_dict()
    c_ora = oracle_mod.Oracle(p).constants(LbmConstants).as_dict()
    assert c_lib == c_ora


def test_invalid_parameters_rejected(gpu_lib):
    import lbmgpu
    for mutate in (lambda p: setattr(p, "nx", 2), lambda p: setattr(p, "Ra", -1.0),
                   lambda p: p.bc_flow.__setitem__(1, 1), lambda p: setattr(p, "precision", 7),
                   lambda p: setattr(p, "Tcold", 1.0)):
        p = rb_params(dim=3, n=16)
        mutate(p)
        with pytest.raises(lbmgpu.LbmError):
            lbmgpu.derive_constants(p)


def test_magnetic_force_only_in_2d_plain_method(gpu_lib, oracle_mod):
    """SideHeatedHa exists in the 2D program only (2DRB.F90:88-92); the FP32/FP16 lag state
    carries F_y only, so those forms refuse it.  The constants follow 2DRB.F90:67, 89-91."""
    import math
    import lbmgpu
    p = rb_params(dim=2, nx=40, ny=20, Ra=1e5)
    p.side_heated_ha, p.Ha, p.phi_deg = 1, 15.0, 30.0
    c = lbmgpu.derive_constants(p)
    assert c.B2sigemarho == (15.0 * 15.0 * c.viscosity) / (c.lengthUnit * c.lengthUnit)
    assert c.phi == 30.0 * (math.acos(-1.0) / 180.0)
    assert (c.sinphi, c.cosphi) == (math.sin(c.phi), math.cos(c.phi))
    assert oracle_mod.Oracle(p).constants(LbmConstants).B2sigemarho == c.B2sigemarho
    for mutate in (lambda q: setattr(q, "precision", 1), lambda q: setattr(q, "precision", 2)):
        q = p.copy()
        mutate(q)
        with pytest.raises(lbmgpu.LbmError):
            lbmgpu.derive_constants(q)
    q3 = rb_params(dim=3, n=16)
    q3.side_heated_ha = 1
    with pytest.raises(lbmgpu.LbmError):
        lbmgpu.derive_constants(q3)


def test_in_place_pattern_accepted_and_smaller(gpu_lib):
    """LBM_PATTERN_AA is a valid pattern for every precision; its device footprint holds one
    population array per lattice (the two-buffer form holds three: A, B and the module
    array) plus face snapshots for periodic axes."""
    import lbmgpu
    for dim in (2, 3):
        for prec in ("fp64", "fp32", "fp16"):
            ab = rb_params(dim=dim, n=64, precision=prec)
            aa = rb_params(dim=dim, n=64, precision=prec, pattern="AA")
            lbmgpu.derive_constants(aa)
            n = ab.nx * ab.ny * (ab.nz if dim == 3 else 1)
            q = 26 if dim == 3 else 14
            es = {"fp64": 8, "fp32": 4, "fp16": 2}[prec]
            saved = lbmgpu.footprint(ab) - lbmgpu.footprint(aa)
            lag = 0 if prec == "fp64" else 4 * n * (4 if dim == 3 else 3)
            faces = es * (19 + 7 if dim == 3 else 9 + 5) * ab.ny if dim == 2 else 0  # 2D cells are x-periodic
            assert saved == 2 * es * q * n + lag - faces, (dim, prec)


def header_constants():
    """#define LBM_* integer constants of the C header."""
    out = {}
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        for m in re.finditer(r"^#define\s+(LBM_[A-Z0-9_]+)\s+(-?\d+)\b", open(h).read(), re.M):
            out[m.group(1)] = int(m.group(2))
    return out


def test_python_and_fortran_constants_match_the_header():
    """Every LBM_* constant the Python package or the Fortran module defines has the header's
    value (the three copies are written by hand)."""
    import lbmgpu
    import lbmgpu.abi as abi
    hdr = header_constants()
    assert "LBM_OPT_WIDE_INDEX" in hdr and "LBM_OPT_ROWS" in hdr
    py = {k: getattr(mod, k) for mod in (lbmgpu, abi) for k in dir(mod) if k.startswith("LBM_")
          and isinstance(getattr(mod, k), int)}
    wrong = {k: (v, hdr[k]) for k, v in py.items() if k in hdr and v != hdr[k]}
    assert not wrong, wrong
    for k in [k for k in hdr if k.startswith("LBM_OPT_")]:
        assert k in py, "lbmgpu lacks %s" % k
    fortran = glob.glob(os.path.join(ROOT, "-2d-3d-_gb300", "fortran", "*.F90"))
    assert fortran
    text = open(fortran[0]).read()
    fvals = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(LBM_[A-Z0-9_]+)\s*=\s*(-?\d+)", text)}
    wrong = {k: (v, hdr[k]) for k, v in fvals.items() if k in hdr and v != hdr[k]}
    assert not wrong, wrong
    for k in [k for k in hdr if k.startswith("LBM_OPT_")]:
        assert k in fvals, "the Fortran module lacks %s" % k
