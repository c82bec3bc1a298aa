"""ctypes wrapper of the CPU oracle (test infrastructure only).

Imported by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, always as
the checker or the timed CPU restatement of the reference; never by the product library.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liblbmoracle.so")
SOURCES = [os.path.join(HERE, "lbm_oracle.cpp")]
HEADERS = [os.path.join(HERE, "lbm_oracle.h"), os.path.join(HERE, "..", "include", "lbm_gpu.h")]

# -ffp-contract=off: the reference's expressions are evaluated one rounding per operation
# (gfortran without -ffast-math); GCC on aarch64 would otherwise fuse a*b+c into an FMA.
CXXFLAGS = ["-std=c++17", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
            "-Wall", "-Wextra"]


def build(force=False, quiet=True):
    """Compile the oracle into oracle/_build/liblbmoracle.so (g++, a few seconds)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SOURCES + HEADERS)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["g++"] + CXXFLAGS + ["-o", tmp] + SOURCES
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB_PATH)
    if not quiet:
        print("built", LIB_PATH, file=sys.stderr)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = C.CDLL(path)
        vp, i32, dp = C.c_void_p, C.c_int, C.POINTER(C.c_double)
        L.ora_create.argtypes = [vp, C.POINTER(vp)]
        L.ora_create.restype = i32
        L.ora_destroy.argtypes = [vp]
        L.ora_destroy.restype = None
        L.ora_constants.argtypes = [vp, vp]
        L.ora_set_threads.argtypes = [i32]
        L.ora_set_threads.restype = i32
        L.ora_initial.argtypes = [vp]
        for n in ("collision", "streaming", "bounceback", "macro",
                  "collisionT", "streamingT", "bouncebackT", "macroT"):
            fn = getattr(L, "ora_" + n)
            fn.argtypes = [vp]
            fn.restype = None
        L.ora_step.argtypes = [vp, C.c_longlong]
        L.ora_step.restype = None
        L.ora_reconstruct_macro_from_fg.argtypes = [vp]
        L.ora_reconstruct_macro_from_fg.restype = i32
        L.ora_check.argtypes = [vp, dp, dp]
        L.ora_calNuRe.argtypes = [vp, dp, dp]
        L.ora_RBcalc_Nu_global.argtypes = [vp, dp]
        L.ora_RBcalc_Nu_wall_avg.argtypes = [vp, vp]
        L.ora_SideHeatedcalc_Nu_global.argtypes = [vp, dp]
        L.ora_SideHeatedcalc_Nu_wall_avg.argtypes = [vp, vp]
        L.ora_mid_max.argtypes = [vp, i32, i32, vp]
        L.ora_get_state.argtypes = [vp, i32, dp, C.c_size_t]
        L.ora_set_state.argtypes = [vp, i32, dp, C.c_size_t]
        L.ora_transform_matrices.argtypes = [i32, dp, dp]
        _lib = L
    return _lib


def set_threads(n):
    return lib().ora_set_threads(int(n))


def transform_matrices(lattice):
    q = int(lattice)
    M = np.zeros((q, q))
    Minv = np.zeros((q, q))
    st = lib().ora_transform_matrices(q, M.ctypes.data_as(C.POINTER(C.c_double)),
                                      Minv.ctypes.data_as(C.POINTER(C.c_double)))
    if st != 0:
        raise ValueError("bad lattice %d" % q)
    return M, Minv


class Oracle:
    """The reference's module state and subroutines, on the CPU, in Fortran layout."""

    def __init__(self, params):
        self.params = params.copy()
        h = C.c_void_p()
        st = lib().ora_create(C.byref(self.params), C.byref(h))
        if st != 0:
            raise ValueError("oracle rejected parameters (status %d)" % st)
        self._h = h

    def close(self):
        if self._h:
            lib().ora_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def constants(self, struct_type):
        c = struct_type()
        lib().ora_constants(self._h, C.byref(c))
        return c

    def initial(self):
        lib().ora_initial(self._h)

    def collision(self): lib().ora_collision(self._h)
    def streaming(self): lib().ora_streaming(self._h)
    def bounceback(self): lib().ora_bounceback(self._h)
    def macro(self): lib().ora_macro(self._h)
    def collisionT(self): lib().ora_collisionT(self._h)
    def streamingT(self): lib().ora_streamingT(self._h)
    def bouncebackT(self): lib().ora_bouncebackT(self._h)
    def macroT(self): lib().ora_macroT(self._h)

    def step(self, n=1):
        lib().ora_step(self._h, int(n))

    def reconstruct_macro_from_fg(self):
        """Restart reconstruction (2DRB.F90:1144-1200, 3DRB.F90:1392-1463); True if some rho <= 0."""
        return bool(lib().ora_reconstruct_macro_from_fg(self._h))

    def check(self):
        a, b = C.c_double(), C.c_double()
        st = lib().ora_check(self._h, C.byref(a), C.byref(b))
        return a.value, b.value, st

    def calNuRe(self):
        a, b = C.c_double(), C.c_double()
        st = lib().ora_calNuRe(self._h, C.byref(a), C.byref(b))
        return a.value, b.value, st

    def RBcalc_Nu_global(self):
        a = C.c_double()
        st = lib().ora_RBcalc_Nu_global(self._h, C.byref(a))
        return a.value, st

    def RBcalc_Nu_wall_avg(self, struct_type):
        w = struct_type()
        st = lib().ora_RBcalc_Nu_wall_avg(self._h, C.byref(w))
        return w, st

    def SideHeatedcalc_Nu_global(self):
        a = C.c_double()
        st = lib().ora_SideHeatedcalc_Nu_global(self._h, C.byref(a))
        return a.value, st

    def SideHeatedcalc_Nu_wall_avg(self, struct_type):
        w = struct_type()
        st = lib().ora_SideHeatedcalc_Nu_wall_avg(self._h, C.byref(w))
        return w.as_dict(), st

    def mid_max(self, comp, rb, struct_type):
        """comp 0/1/2 = u/v/w; rb: the RB form of the 2D u line."""
        m = struct_type()
        st = lib().ora_mid_max(self._h, int(comp), int(rb), C.byref(m))
        return m.as_dict(), st

    def get(self, field_id, shape):
        a = np.empty(shape, dtype=np.float64)
        st = lib().ora_get_state(self._h, int(field_id), a.ctypes.data_as(C.POINTER(C.c_double)), a.size)
        if st != 0:
            raise ValueError("oracle get_state(%d) failed: %d" % (field_id, st))
        return a

    def set(self, field_id, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        st = lib().ora_set_state(self._h, int(field_id), a.ctypes.data_as(C.POINTER(C.c_double)), a.size)
        if st != 0:
            raise ValueError("oracle set_state(%d) failed: %d" % (field_id, st))
