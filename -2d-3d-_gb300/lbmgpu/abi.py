"""ctypes mirror of include/lbm_gpu.h (structs, constants, signatures).

The structs follow the C layout exactly (natural alignment), so the same objects can be
handed to any library that takes `const lbm_params*`.
"""
import ctypes as C
import math

LBM_OK, LBM_ERR_PARAM, LBM_ERR_CUDA, LBM_ERR_OOM, LBM_ERR_DIVERGED, LBM_ERR_TIMEOUT, LBM_ERR_STATE = range(7)
STATUS_NAMES = {0: "LBM_OK", 1: "LBM_ERR_PARAM", 2: "LBM_ERR_CUDA", 3: "LBM_ERR_OOM",
                4: "LBM_ERR_DIVERGED", 5: "LBM_ERR_TIMEOUT", 6: "LBM_ERR_STATE", 7: "LBM_ERR_TOO_LARGE",
                8: "LBM_ERR_IO"}
LBM_ERR_IO = 8
LBM_BACKUP_REFERENCE, LBM_BACKUP_CONTINUE = 0, 1
LBM_RELOAD_REFERENCE, LBM_RELOAD_CONTINUE, LBM_RELOAD_AUTO = 0, 1, 2

LBM_CELL_RB, LBM_CELL_SIDE = 0, 1
LBM_BC_NOSLIP, LBM_BC_PERIODIC = 0, 1
LBM_BCT_CONST, LBM_BCT_ADIABATIC, LBM_BCT_PERIODIC = 0, 1, 2
LBM_FP64, LBM_FP32, LBM_FP16 = 0, 1, 2
LBM_PATTERN_AB, LBM_PATTERN_AA = 0, 1
LBM_ARITH_REFERENCE, LBM_ARITH_FIXED = 0, 1

FIELDS = {
    "f": 0, "g": 1, "rho": 2, "u": 3, "v": 4, "w": 5, "T": 6,
    "Bx_prev": 7, "By_prev": 8, "Bz_prev": 9, "Fx": 10, "Fy": 11, "f_post": 12, "g_post": 13,
}
PRECISIONS = {"fp64": LBM_FP64, "fp32": LBM_FP32, "fp16": LBM_FP16}
# "fp64x": FP64 handle with the fixed arithmetic (FP64 accuracy on the integer pipes)
PRECISION_NAMES = {"fp64": (LBM_FP64, LBM_ARITH_REFERENCE), "fp64x": (LBM_FP64, LBM_ARITH_FIXED),
                   "fp32": (LBM_FP32, LBM_ARITH_REFERENCE), "fp16": (LBM_FP16, LBM_ARITH_REFERENCE)}


class LbmParams(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("Ra", C.c_double), ("Pr", C.c_double), ("Mach", C.c_double),
        ("Thot", C.c_double), ("Tcold", C.c_double),
        ("cell", C.c_int32), ("bc_flow", C.c_int32 * 3), ("bc_thermal", C.c_int32 * 3),
        ("use_g", C.c_int32), ("legacy_thermal", C.c_int32),
        ("precision", C.c_int32), ("pattern", C.c_int32),
        ("seed", C.c_uint64), ("noise_amp", C.c_double),
        ("side_heated_ha", C.c_int32), ("arith", C.c_int32), ("Ha", C.c_double), ("phi_deg", C.c_double),
    ]

    def copy(self):
        out = LbmParams()
        C.pointer(out)[0] = self
        return out

    def describe(self):
        return {
            "dim": self.dim, "nx": self.nx, "ny": self.ny, "nz": self.nz, "Ra": self.Ra, "Pr": self.Pr,
            "Mach": self.Mach,
            "precision": "fp64x" if self.arith == LBM_ARITH_FIXED else {v: k for k, v in PRECISIONS.items()}[self.precision],
            "pattern": "AA" if self.pattern == LBM_PATTERN_AA else "AB",
        }


class LbmConstants(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "lengthUnit", "Tref", "tauf", "viscosity", "diffusivity", "paraA",
        "gBeta", "timeUnit", "velocityUnit", "heatFluxScale", "velocityScaleCompare",
        "Snu", "Sq", "Se", "Seps", "Spi", "Sm",
        "taug", "Qk", "Qnu", "SG", "thermalGeqCoeff", "cs2T", "omegaT0", "omegaT1",
        "B2sigemarho", "phi", "sinphi", "cosphi")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class LbmNuWall(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "Nu_hot", "Nu_cold", "Nu_middle", "Nu_hot_max", "Nu_hot_max_position",
        "Nu_hot_min", "Nu_hot_min_position")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class LbmPsiSummary(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("psi_center", "psi_center_abs", "psi_abs_max", "x_at_max", "y_at_max",
                                          "psi_center_abs_fine")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class LbmMidMax(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("value", "pos1", "pos2", "mid")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


def rb_params(dim=3, n=None, nx=None, ny=None, nz=None, Ra=1e7, Pr=0.71, U=0.1, Mach=None,
              precision="fp64", pattern="AB", seed=20261203, noise_amp=1e-3,
              periodic_x=None, legacy_thermal=False, use_g=True):
    """Rayleigh-Benard cell parameters in the reference's terms.

    U is the free-fall velocity in lattice units; the reference's Mach is U*sqrt(3)
    (tauf = 0.5 + Mach*L*sqrt(3Pr/Ra) gives nu = U*H*sqrt(Pr/Ra)).  2D cells default to
    the reference's 2DRB.F90 switches (x periodic); 3D cells to no-slip everywhere with
    adiabatic side walls.
    """
    p = LbmParams()
    p.dim = dim
    if dim == 2:
        p.ny = ny if ny is not None else (n if n is not None else 128)
        p.nx = nx if nx is not None else 2 * p.ny
        p.nz = 1
    else:
        n = n if n is not None else 64
        p.nx = nx if nx is not None else n
        p.ny = ny if ny is not None else n
        p.nz = nz if nz is not None else n
    p.Ra, p.Pr = float(Ra), float(Pr)
    p.Mach = float(Mach) if Mach is not None else float(U) * math.sqrt(3.0)
    p.Thot, p.Tcold = 0.5, -0.5
    p.cell = LBM_CELL_RB
    if periodic_x is None:
        periodic_x = (dim == 2)
    p.bc_flow[0] = LBM_BC_PERIODIC if periodic_x else LBM_BC_NOSLIP
    p.bc_flow[1] = LBM_BC_NOSLIP
    p.bc_flow[2] = LBM_BC_NOSLIP
    p.bc_thermal[0] = LBM_BCT_PERIODIC if periodic_x else LBM_BCT_ADIABATIC
    p.bc_thermal[1] = LBM_BCT_CONST
    p.bc_thermal[2] = LBM_BCT_ADIABATIC
    p.use_g = 1 if use_g else 0
    p.legacy_thermal = 1 if legacy_thermal else 0
    if isinstance(precision, str):
        p.precision, p.arith = PRECISION_NAMES[precision]
    else:
        p.precision, p.arith = int(precision), LBM_ARITH_REFERENCE
    p.pattern = LBM_PATTERN_AA if str(pattern).upper() == "AA" else LBM_PATTERN_AB
    p.seed = int(seed)
    p.noise_amp = float(noise_amp)
    return p


def field_size(p, field):
    ncell = p.nx * p.ny * (p.nz if p.dim == 3 else 1)
    q, qt = (19, 7) if p.dim == 3 else (9, 5)
    f = FIELDS[field] if isinstance(field, str) else field
    if f in (0, 12):
        return q * ncell
    if f in (1, 13):
        return qt * ncell
    return ncell


def field_shape(p, field):
    """numpy shape (C order) of a field in the reference's Fortran layout."""
    nz = p.nz if p.dim == 3 else 1
    q, qt = (19, 7) if p.dim == 3 else (9, 5)
    f = FIELDS[field] if isinstance(field, str) else field
    lead = {0: q, 12: q, 1: qt, 13: qt}.get(f)
    base = (nz, p.ny, p.nx) if p.dim == 3 else (p.ny, p.nx)
    return base + ((lead,) if lead else ())
