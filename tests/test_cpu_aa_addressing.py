"""In-place (AA) addressing, checked on the host: the device helpers that decide where a
cell reads and writes (pull_flow_w, pull_thermal_w, aa_push, aa_local_thermal,
aa_face_index; csrc/lbm_device.cuh) are compiled as C++ and driven through in-place sweeps
against the two-buffer pull on 18 boundary combinations (aa_addressing_check.cpp)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_in_place_addressing(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "aa_addressing_check")
    cmd = [cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "-2d-3d-_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
           "-o", exe, os.path.join(HERE, "aa_addressing_check.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
