"""lbmgpu - Python mirror of the reference's subroutine surface over the C ABI.

The reference (2DRB/2DRB.F90, 2DRB/3DRB.F90) is a Fortran program whose hot path is a
fixed sequence of argument-less subroutines acting on module arrays:

    initial; do: collision, streaming, bounceback, macro,
                 collisionT, streamingT, bouncebackT, macroT; check every 2000 steps
    RBcalc_Nu_global, RBcalc_Nu_wall_avg, calNuRe at the end

`Lattice` keeps that surface (same names, same meaning) on top of liblbmgpu.so, whose
kernels are hand-written CUDA for sm_103a.  There is no CPU fallback: every method calls
the library, and a missing library or GPU raises.
"""
import ctypes as C
import os

import numpy as np

from .abi import (FIELDS, LBM_BACKUP_CONTINUE, LBM_BACKUP_REFERENCE, LBM_FP64, LBM_OK, LBM_RELOAD_AUTO,
                  LBM_RELOAD_CONTINUE, LBM_RELOAD_REFERENCE, STATUS_NAMES, LbmConstants, LbmMidMax, LbmNuWall,
                  LbmParams, field_shape, field_size, rb_params)

__all__ = ["Lattice", "Ensemble", "LbmError", "LbmDiverged", "LbmParams", "rb_params", "load_library",
           "library_path", "params_default", "derive_constants", "footprint", "FIELDS"]

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_NAME = "liblbmgpu.so"

# Every entry point of include/lbm_gpu.h with its ctypes signature.
_vp, _i32, _i64, _dp, _sz = C.c_void_p, C.c_int, C.c_int64, C.POINTER(C.c_double), C.c_size_t
SIGNATURES = {
    "lbm_params_default": ([_i32, _vp], _i32),
    "lbm_derive_constants": ([_vp, _vp], _i32),
    "lbm_create": ([_vp, _i32, C.POINTER(_vp)], _i32),
    "lbm_destroy": ([_vp], _i32),
    "lbm_initial": ([_vp], _i32),
    "lbm_last_error": ([_vp], C.c_char_p),
    "lbm_status_string": ([_i32], C.c_char_p),
    "lbm_get_constants": ([_vp, _vp], _i32),
    "lbm_itc": ([_vp], _i64),
    "lbm_sync": ([_vp], _i32),
    "lbm_collision": ([_vp], _i32),
    "lbm_streaming": ([_vp], _i32),
    "lbm_bounceback": ([_vp], _i32),
    "lbm_macro": ([_vp], _i32),
    "lbm_collisionT": ([_vp], _i32),
    "lbm_streamingT": ([_vp], _i32),
    "lbm_bouncebackT": ([_vp], _i32),
    "lbm_macroT": ([_vp], _i32),
    "lbm_step": ([_vp, _i64], _i32),
    "lbm_check": ([_vp, _dp, _dp], _i32),
    "lbm_check_log": ([_vp, C.c_char_p, _i32, _dp, _dp], _i32),
    "lbm_append_convergence_tecplot": ([_vp, C.c_char_p, _i64, C.c_double, C.c_double], _i32),
    "lbm_append_convergence_master_tecplot": ([_vp, C.c_char_p, C.c_char_p, _i64, C.c_double, C.c_double], _i32),
    "lbm_case_tag": ([_vp, C.c_char_p, _sz], _i32),
    "lbm_append_convergence_tecplot_host": ([C.c_char_p, _i32, _i32, _i64, C.c_double, C.c_double], _i32),
    "lbm_append_convergence_master_tecplot_host": ([C.c_char_p, _i32, _i32, C.c_char_p, _i64, C.c_double, C.c_double],
                                                   _i32),
    "lbm_convergence_line": ([_i64, C.c_double, C.c_double, C.c_char_p, _sz], _i32),
    "lbm_format_fortran_es": ([C.c_double, _i32, _i32, _i32, C.c_char_p, _sz], _i32),
    "lbm_calNuRe": ([_vp, _dp, _dp], _i32),
    "lbm_RBcalc_Nu_global": ([_vp, _dp], _i32),
    "lbm_RBcalc_Nu_wall_avg": ([_vp, _vp], _i32),
    "lbm_get_state": ([_vp, _i32, _dp, _sz], _i32),
    "lbm_set_state": ([_vp, _i32, _dp, _sz], _i32),
    "lbm_get_stream": ([_vp, C.POINTER(_vp)], _i32),
    "lbm_time_kernels": ([_vp, _i64, _dp, _dp], _i32),
    "lbm_selftest_wait_timeout": ([_vp, _i64], _i32),
    "lbm_set_option": ([_vp, _i32, _i32], _i32),
    "lbm_footprint": ([_vp, C.POINTER(_sz)], _i32),
    "lbm_ensemble_create": ([_i32, C.POINTER(_vp)], _i32),
    "lbm_ensemble_destroy": ([_vp], _i32),
    "lbm_ensemble_add": ([_vp, _vp], _i32),
    "lbm_ensemble_remove": ([_vp, _vp], _i32),
    "lbm_ensemble_size": ([_vp], _i32),
    "lbm_ensemble_step": ([_vp, _i64], _i32),
    "lbm_ensemble_sync": ([_vp], _i32),
    "lbm_ensemble_get_stream": ([_vp, C.POINTER(_vp)], _i32),
    "lbm_ensemble_last_error": ([_vp], C.c_char_p),
    "lbm_ensemble_autotune": ([_vp, _i32, C.POINTER(_i32), C.POINTER(_i32), C.POINTER(_i32)], _i32),
    "lbm_ensemble_configure": ([_vp, _i32, _i32, _i32, _i32], _i32),
    "lbm_ensemble_get_launch": ([_vp, C.POINTER(_i32), C.POINTER(_i32), C.POINTER(_i32), C.POINTER(_i32)], _i32),
    "lbm_SideHeatedcalc_Nu_global": ([_vp, _dp], _i32),
    "lbm_SideHeatedcalc_Nu_wall_avg": ([_vp, _vp], _i32),
    "lbm_SideHeatedcalc_umid_max": ([_vp, _vp], _i32),
    "lbm_SideHeatedcalc_vmid_max": ([_vp, _vp], _i32),
    "lbm_SideHeatedcalc_wmid_max": ([_vp, _vp], _i32),
    "lbm_RBcalc_umid_max": ([_vp, _vp], _i32),
    "lbm_RBcalc_vmid_max": ([_vp, _vp], _i32),
    "lbm_RBcalc_wmid_max": ([_vp, _vp], _i32),
    "lbm_get_params": ([_vp, _vp], _i32),
    "lbm_output_binary": ([_vp, C.c_char_p], _i32),
    "lbm_output_Tecplot": ([_vp, C.c_char_p, _i64], _i32),
    "lbm_calc_psi_vort_and_output": ([_vp, C.c_char_p, _i64, _i32, _vp], _i32),
    "lbm_output_binary_host": ([C.c_char_p, _i32, _i32, _i32, _i32, C.c_double, _dp, _dp, _dp, _dp, _dp], _i32),
    "lbm_tecplot_fields_2d": ([C.c_char_p, _i32, _i32, C.c_double, C.c_double, _dp, _dp, _dp], _i32),
    "lbm_tecplot_full_3d": ([C.c_char_p, _i32, _i32, _i32, C.c_double, _dp, _dp, _dp, _dp], _i32),
    "lbm_tecplot_midplane_3d": ([C.c_char_p, _i32, _i32, _i32, _i32, C.c_double, C.c_double, _dp, _dp, _dp, _dp],
                                _i32),
    "lbm_tecplot_midplane_stream_3d": ([C.c_char_p, _i32, _i32, _i32, _i32, C.c_double, C.c_double, _dp, _dp, _dp],
                                       _i32),
    "lbm_psi_vort_2d": ([_i32, _i32, C.c_double, C.c_double, _dp, _dp, _dp, _dp], _i32),
    "lbm_tecplot_psi_vort_2d": ([C.c_char_p, _i32, _i32, C.c_double, _dp, _dp], _i32),
    "lbm_psi_center_2d": ([_i32, _i32, C.c_double, _dp, _dp], _i32),
    "lbm_psi_absmax_fine_spline": ([_i32, _i32, C.c_double, _dp, _i32, _dp, _dp, _dp, _dp], _i32),
    "lbm_backupData": ([_vp, C.c_char_p, _i32], _i32),
    "lbm_reload": ([_vp, C.c_char_p, _i32], _i32),
    "lbm_reload_form": ([_vp], _i32),
    "lbm_fortran_record_write": ([C.c_char_p, _i32, _vp, _sz], _i32),
    "lbm_fortran_record_read": ([C.c_char_p, C.c_uint64, _vp, _sz, C.POINTER(_sz), C.POINTER(C.c_uint64)], _i32),
    "lbm_fortran_set_subrecord_limit": ([_sz], _i32),
}
LBM_OPT_SINGLE_KERNEL = 1
LBM_OPT_KCHUNK = 2
LBM_OPT_PAIRS = 3
LBM_OPT_STAGED = 4
LBM_OPT_FP16_ROUNDING = 5  # FP16 storage: 1 stochastic rounding (default), 0 nearest
LBM_OPT_WIDE_INDEX = 8     # fixed arithmetic: 64-bit indices in every kernel (1) or 32-bit ones where they fit (0)
LBM_OPT_ROWS = 7           # FP32/FP16 two-buffer steps: interior-row and face-row launches (1) or one cell per thread
LBM_OPT_HOST_DIRECT = 6    # state transfer on the caller's host arrays: bit 0 set_state reads, bit 1 get_state writes

_lib = None


def library_path():
    return os.path.join(_PKG, LIB_NAME)


def load_library(path=None):
    """Load liblbmgpu.so from the package directory (built in-tree by lbmgpu.build), or from
    the path in the environment variable LBMGPU_LIBRARY when it is set."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or os.environ.get("LBMGPU_LIBRARY") or library_path()
    if not os.path.exists(p):
        raise RuntimeError("%s is not built; run lbmgpu.build.build() (nvcc, sm_103a)" % p)
    lib = C.CDLL(p)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


class LbmError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


class LbmDiverged(LbmError):
    pass


def params_default(dim):
    p = LbmParams()
    st = load_library().lbm_params_default(int(dim), C.byref(p))
    if st != LBM_OK:
        raise LbmError(st, "lbm_params_default")
    return p


def derive_constants(params):
    c = LbmConstants()
    st = load_library().lbm_derive_constants(C.byref(params), C.byref(c))
    if st != LBM_OK:
        raise LbmError(st, "invalid parameters")
    return c


def footprint(params):
    """Device bytes a Lattice with these parameters allocates."""
    b = C.c_size_t()
    st = load_library().lbm_footprint(C.byref(params), C.byref(b))
    if st != LBM_OK:
        raise LbmError(st, "invalid parameters")
    return int(b.value)


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Lattice:
    """One lattice resident on one GPU; methods are the reference's subroutines."""

    def __init__(self, params, device=0):
        self.lib = load_library()
        self.params = params.copy()
        h = C.c_void_p()
        st = self.lib.lbm_create(C.byref(self.params), int(device), C.byref(h))
        if st != LBM_OK:
            raise LbmError(st, "lbm_create failed (parameters, device %d or memory)" % device)
        self._h = h

    # -- lifecycle -------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self.lib.lbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _ck(self, st, what):
        if st != LBM_OK:
            msg = self.lib.lbm_last_error(self._h)
            msg = msg.decode() if msg else what
            cls = LbmDiverged if st == 4 else LbmError
            raise cls(st, "%s: %s" % (what, msg))

    @property
    def itc(self):
        return int(self.lib.lbm_itc(self._h))

    def constants(self):
        c = LbmConstants()
        self._ck(self.lib.lbm_get_constants(self._h, C.byref(c)), "lbm_get_constants")
        return c.as_dict()

    def sync(self):
        self._ck(self.lib.lbm_sync(self._h), "lbm_sync")

    # -- the reference's subroutines ---------------------------------------------------
    def initial(self):
        self._ck(self.lib.lbm_initial(self._h), "initial")

    def collision(self): self._ck(self.lib.lbm_collision(self._h), "collision")
    def streaming(self): self._ck(self.lib.lbm_streaming(self._h), "streaming")
    def bounceback(self): self._ck(self.lib.lbm_bounceback(self._h), "bounceback")
    def macro(self): self._ck(self.lib.lbm_macro(self._h), "macro")
    def collisionT(self): self._ck(self.lib.lbm_collisionT(self._h), "collisionT")
    def streamingT(self): self._ck(self.lib.lbm_streamingT(self._h), "streamingT")
    def bouncebackT(self): self._ck(self.lib.lbm_bouncebackT(self._h), "bouncebackT")
    def macroT(self): self._ck(self.lib.lbm_macroT(self._h), "macroT")

    def stage_step(self):
        """One iteration of the reference's loop body through the eight stage kernels."""
        for s in (self.collision, self.streaming, self.bounceback, self.macro,
                  self.collisionT, self.streamingT, self.bouncebackT, self.macroT):
            s()

    def step(self, nsteps=1):
        """nsteps iterations with the fused kernels (asynchronous)."""
        self._ck(self.lib.lbm_step(self._h, int(nsteps)), "lbm_step")

    def check(self):
        a, b = C.c_double(), C.c_double()
        self._ck(self.lib.lbm_check(self._h, C.byref(a), C.byref(b)), "check")
        return a.value, b.value

    def check_log(self, directory=".", echo=False):
        """check as the reference runs it: the errors, appended to convergence[3D].plt and
        (under case_tag()) convergence_all[_3D].plt in `directory`, echoed when echo."""
        a, b = C.c_double(), C.c_double()
        self._ck(self.lib.lbm_check_log(self._h, os.fsencode(directory), 1 if echo else 0, C.byref(a), C.byref(b)),
                 "check_log")
        return a.value, b.value

    def case_tag(self):
        """The reference's caseTag string of this lattice (Ra, sizes, useG, legacy switch)."""
        buf = C.create_string_buffer(256)
        self._ck(self.lib.lbm_case_tag(self._h, buf, 256), "case_tag")
        return buf.value.decode()

    def calNuRe(self):
        a, b = C.c_double(), C.c_double()
        self._ck(self.lib.lbm_calNuRe(self._h, C.byref(a), C.byref(b)), "calNuRe")
        return a.value, b.value

    def RBcalc_Nu_global(self):
        a = C.c_double()
        self._ck(self.lib.lbm_RBcalc_Nu_global(self._h, C.byref(a)), "RBcalc_Nu_global")
        return a.value

    def RBcalc_Nu_wall_avg(self):
        w = LbmNuWall()
        self._ck(self.lib.lbm_RBcalc_Nu_wall_avg(self._h, C.byref(w)), "RBcalc_Nu_wall_avg")
        return w.as_dict()

    def SideHeatedcalc_Nu_global(self):
        a = C.c_double()
        self._ck(self.lib.lbm_SideHeatedcalc_Nu_global(self._h, C.byref(a)), "SideHeatedcalc_Nu_global")
        return a.value

    def SideHeatedcalc_Nu_wall_avg(self):
        w = LbmNuWall()
        self._ck(self.lib.lbm_SideHeatedcalc_Nu_wall_avg(self._h, C.byref(w)), "SideHeatedcalc_Nu_wall_avg")
        return w.as_dict()

    def _mid_max(self, name):
        m = LbmMidMax()
        self._ck(getattr(self.lib, "lbm_" + name)(self._h, C.byref(m)), name)
        return m.as_dict()

    def SideHeatedcalc_umid_max(self): return self._mid_max("SideHeatedcalc_umid_max")
    def SideHeatedcalc_vmid_max(self): return self._mid_max("SideHeatedcalc_vmid_max")
    def SideHeatedcalc_wmid_max(self): return self._mid_max("SideHeatedcalc_wmid_max")
    def RBcalc_umid_max(self): return self._mid_max("RBcalc_umid_max")
    def RBcalc_vmid_max(self): return self._mid_max("RBcalc_vmid_max")
    def RBcalc_wmid_max(self): return self._mid_max("RBcalc_wmid_max")

    # -- measurement ----------------------------------------------------------------------
    def stream_handle(self):
        """The cudaStream_t the handle enqueues on (as an integer), e.g. for torch.cuda.ExternalStream."""
        s = C.c_void_p()
        self._ck(self.lib.lbm_get_stream(self._h, C.byref(s)), "lbm_get_stream")
        return s.value or 0

    def set_option(self, option, value):
        """LBM_OPT_SINGLE_KERNEL (0/1) or LBM_OPT_KCHUNK (z planes per block of the fused kernel)."""
        self._ck(self.lib.lbm_set_option(self._h, int(option), int(value)), "lbm_set_option")

    def time_kernels(self, nsteps):
        """Mean device ms per launch of the (flow, thermal) fused kernels over nsteps steps."""
        a, b = C.c_double(), C.c_double()
        self._ck(self.lib.lbm_time_kernels(self._h, int(nsteps), C.byref(a), C.byref(b)), "lbm_time_kernels")
        return a.value, b.value

    # -- restart files (backupData / loadInitField = 1) --------------------------------------
    def backupData(self, path, continuation=True):
        """Write the reference's restart file (f and g records, 3DRB.F90:1638-1665); with
        continuation=True also the records that make a reload bit-continuous."""
        flags = LBM_BACKUP_CONTINUE if continuation else LBM_BACKUP_REFERENCE
        self._ck(self.lib.lbm_backupData(self._h, os.fsencode(path), flags), "backupData")

    def reload(self, path, mode="auto"):
        """Replace the state from a restart file.  mode: "reference" (f, g and
        reconstruct_macro_from_fg), "continue" (bit-continuous records required) or "auto".
        Returns the form used: "reference" or "continue"."""
        m = {"reference": LBM_RELOAD_REFERENCE, "continue": LBM_RELOAD_CONTINUE, "auto": LBM_RELOAD_AUTO}[mode]
        self._ck(self.lib.lbm_reload(self._h, os.fsencode(path), m), "reload")
        return "continue" if self.lib.lbm_reload_form(self._h) == 1 else "reference"

    # -- snapshot writers (output_binary, output_Tecplot, calc_psi_vort_and_output) ----
    def output_binary(self, path):
        """The reference's output_binary file: records of (L/kappa) u, v[, w], T, rho."""
        self._ck(self.lib.lbm_output_binary(self._h, os.fsencode(path)), "output_binary")

    def output_Tecplot(self, prefix, number=0):
        """The reference's Tecplot files <prefix>-...<number, 12 digits>.plt (one in 2D, seven in 3D)."""
        self._ck(self.lib.lbm_output_Tecplot(self._h, os.fsencode(prefix), int(number)), "output_Tecplot")

    def calc_psi_vort_and_output(self, prefix=None, number=0, fine_per_unit=10000):
        """2D stream function / vorticity: writes <prefix>-psiVort-<n>.plt (unless prefix is
        None) and returns the centre value and the fine-grid maximum of |psi|."""
        from .abi import LbmPsiSummary
        out = LbmPsiSummary()
        pre = os.fsencode(prefix) if prefix is not None else None
        self._ck(self.lib.lbm_calc_psi_vort_and_output(self._h, pre, int(number), int(fine_per_unit), C.byref(out)),
                 "calc_psi_vort_and_output")
        return out.as_dict()

    # -- state transfer (Fortran layout) ------------------------------------------------
    def get_state(self, field):
        fid = FIELDS[field] if isinstance(field, str) else int(field)
        a = np.empty(field_shape(self.params, fid), dtype=np.float64)
        self._ck(self.lib.lbm_get_state(self._h, fid, _dptr(a), a.size), "get_state(%s)" % field)
        return a

    def set_state(self, field, arr):
        fid = FIELDS[field] if isinstance(field, str) else int(field)
        a = np.ascontiguousarray(arr, dtype=np.float64)
        if a.size != field_size(self.params, fid):
            raise ValueError("set_state(%s): expected %d values, got %d" % (field, field_size(self.params, fid), a.size))
        self._ck(self.lib.lbm_set_state(self._h, fid, _dptr(a), a.size), "set_state(%s)" % field)


class Ensemble:
    """Many FP32/FP16 lattices advanced together: one flow and one thermal launch per step
    over a packed tile table of all members (the batched form)."""

    def __init__(self, device=0):
        self.lib = load_library()
        h = C.c_void_p()
        st = self.lib.lbm_ensemble_create(int(device), C.byref(h))
        if st != LBM_OK:
            raise LbmError(st, "lbm_ensemble_create")
        self._h = h
        self.members = []

    def _ck(self, st, what):
        if st != LBM_OK:
            msg = self.lib.lbm_ensemble_last_error(self._h)
            raise LbmError(st, "%s: %s" % (what, msg.decode() if msg else ""))

    def add(self, lattice):
        self._ck(self.lib.lbm_ensemble_add(self._h, lattice._h), "lbm_ensemble_add")
        self.members.append(lattice)

    def remove(self, lattice):
        self._ck(self.lib.lbm_ensemble_remove(self._h, lattice._h), "lbm_ensemble_remove")
        self.members.remove(lattice)

    def __len__(self):
        return int(self.lib.lbm_ensemble_size(self._h))

    def step(self, nsteps):
        self._ck(self.lib.lbm_ensemble_step(self._h, int(nsteps)), "lbm_ensemble_step")

    def sync(self):
        self._ck(self.lib.lbm_ensemble_sync(self._h), "lbm_ensemble_sync")

    def stream_handle(self):
        s = C.c_void_p()
        self._ck(self.lib.lbm_ensemble_get_stream(self._h, C.byref(s)), "lbm_ensemble_get_stream")
        return s.value or 0

    def autotune(self, nsteps=4):
        """Pick the tile / block / grid configuration by timing; members advance meanwhile."""
        b, t, g = C.c_int(), C.c_int(), C.c_int()
        self._ck(self.lib.lbm_ensemble_autotune(self._h, int(nsteps), C.byref(b), C.byref(t), C.byref(g)),
                 "lbm_ensemble_autotune")
        return self.launch()

    def configure(self, block=128, tile_cells=1024, grid_per_sm=8, pairs=1):
        """Set the launch configuration (pairs: bit 0 pairs 2D members with even nx, bit 1
        3D members); the values do not depend on it."""
        self._ck(self.lib.lbm_ensemble_configure(self._h, int(block), int(tile_cells), int(grid_per_sm), int(pairs)),
                 "lbm_ensemble_configure")

    def launch(self):
        b, t, g, p = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self._ck(self.lib.lbm_ensemble_get_launch(self._h, C.byref(b), C.byref(t), C.byref(g), C.byref(p)),
                 "lbm_ensemble_get_launch")
        return {"block": b.value, "tile_cells": t.value, "grid_per_sm": g.value, "pairs": p.value}

    def close(self):
        if getattr(self, "_h", None):
            self.lib.lbm_ensemble_destroy(self._h)
            self._h = None
            self.members = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
