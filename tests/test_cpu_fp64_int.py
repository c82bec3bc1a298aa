"""Integer-pipe binary64 scaling, checked on the host: the exponent add that the plain
method uses for its products with exact powers of two (csrc/lbm_fp64_int.cuh), compiled as
C++ and compared bit for bit with the CPU's IEEE-754 multiplication on 7 M operands plus
the special values (fp64_int_check.cpp).  The device build is compared with the FP64 pipe
by test_gpu_parity.py::test_integer_pipe_arithmetic_matches_fp64."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_power_of_two_scaling_matches_cpu(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "fp64_int_check")
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "-2d-3d-_gb300", "csrc"), "-o", exe,
           os.path.join(HERE, "fp64_int_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
