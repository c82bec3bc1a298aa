"""Build liblbmgpu.so (the C-ABI library) in-tree with nvcc for sm_103a.

Translation units and their floating-point flags:
  lbm_exact.cu  -fmad=false : the plain FP64 method, one rounding per operation as in the reference
  lbm_reduce.cu -fmad=false : FP64 diagnostics, per-cell terms rounded as in the reference
  lbm_fast.cu               : FP32 arithmetic on FP32/FP16 storage, FMA contraction allowed
  lbm_fast_tma.cu           : the same step with population rows staged by bulk copies
  lbm_fast_aa.cu            : the same step in the in-place (AA) access pattern
  lbm_fixed.cu              : the fixed arithmetic of FP64 handles (integer pipes, FP64 accuracy)
  lbm_api.cpp               : host code (-ffp-contract=off for the host-side fits)
  lbm_checkpoint.cpp        : Fortran unformatted sequential records (restart files)
  lbm_output.cpp            : snapshot / Tecplot writers, stream function post-processing
The units compile in parallel; a full build takes well under two minutes.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
BUILD_DIR = os.path.join(ROOT, "_build")
LIB_PATH = os.path.join(PKG_DIR, "liblbmgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", CSRC, "-I", INCLUDE]
UNITS = [
    ("lbm_exact.cu", ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"]),
    ("lbm_reduce.cu", ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"]),
    ("lbm_fast.cu", ["-fmad=true"]),
    ("lbm_fast_tma.cu", ["-fmad=true"]),
    ("lbm_fast_aa.cu", ["-fmad=true"]),
    ("lbm_fused.cu", ["-fmad=true"]),
    ("lbm_ensemble.cu", ["-fmad=true"]),
    ("lbm_api.cpp", []),
    ("lbm_checkpoint.cpp", []),
    ("lbm_output.cpp", []),
    ("lbm_noalloc.cu", ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"]),
    ("lbm_fixed.cu", ["-fmad=false"]),
]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbmgpu.so")


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def up_to_date():
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(p) <= t for p in _sources() + [os.path.abspath(__file__)])


def build(force=False, verbose=False, extra_flags=()):
    """Compile every unit for sm_103a and link the shared library; returns its path."""
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    cc = nvcc()

    def compile_unit(unit):
        name, flags = unit
        src = os.path.join(CSRC, name)
        obj = os.path.join(BUILD_DIR, name + ".o")
        cmd = [cc, "-c", src, "-o", obj] + ARCH + COMMON + flags + list(extra_flags)
        if name.endswith(".cpp"):
            cmd = [cc, "-x", "cu", "-c", src, "-o", obj] + ARCH + COMMON + flags + list(extra_flags)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (name, " ".join(cmd), r.stdout + r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = [cc, "-shared", "-o", tmp] + objs + ARCH + ["-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stdout + r.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
