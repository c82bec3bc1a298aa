"""The snapshot writers on host arrays against the reference's own write statements.

For every step fixture, make_golden.py executed the reference's Tecplot writers
(2DRB.F90 output_Tecplot and output_Tecplot_psi_vort; 3DRB.F90 write_full_fields_plt,
write_midplane_{x,y,z} and write_midplane_stream_{x,y,z}) on the stepped state and kept
the bytes of every `write(unit)` statement.  The library's writers must produce the same
files byte for byte; its 2D stream function, vorticity and centre value must equal the
reference's.  These entry points take host arrays and need no GPU.
"""
import ctypes as C

import numpy as np
import pytest

import golden_cases as gc
from lbmgpu.abi import LBM_OK

MID3 = ["write_midplane_x", "write_midplane_y", "write_midplane_z"]
STREAM3 = ["write_midplane_stream_x", "write_midplane_stream_y", "write_midplane_stream_z"]


def dp(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))


def setup(name, gpu_lib, oracle_mod):
    from lbmgpu.abi import LbmConstants
    meta = gc.cases()[name]
    p = gc.params_for(meta)
    c = oracle_mod.Oracle(p).constants(LbmConstants)
    return meta, p, c, gc.load(name)


@pytest.mark.parametrize("name", sorted(gc.cases()))
def test_tecplot_files_match_reference_bytes(gpu_lib, oracle_mod, tmp_path, name):
    meta, p, c, d = setup(name, gpu_lib, oracle_mod)
    L, vsc = c.lengthUnit, c.velocityScaleCompare
    keep = []

    def arr(k):
        a = np.ascontiguousarray(d["out_" + k], dtype=np.float64)
        keep.append(a)
        return a.ctypes.data_as(C.POINTER(C.c_double))

    f = str(tmp_path / "out.plt")
    if meta["dim"] == 2:
        assert gpu_lib.lbm_tecplot_fields_2d(f.encode(), p.nx, p.ny, L, vsc, arr("u"), arr("v"), arr("T")) == LBM_OK
        assert open(f, "rb").read() == d["plt_fields"].tobytes()
        psi = np.zeros((p.ny, p.nx))
        vort = np.zeros((p.ny, p.nx))
        assert gpu_lib.lbm_psi_vort_2d(p.nx, p.ny, L, vsc, arr("u"), arr("v"), dp(psi), dp(vort)) == LBM_OK
        assert np.array_equal(psi, d["psi_psi"]) and np.array_equal(vort, d["psi_vort"])
        assert gpu_lib.lbm_tecplot_psi_vort_2d(f.encode(), p.nx, p.ny, L, dp(psi), dp(vort)) == LBM_OK
        assert open(f, "rb").read() == d["plt_psiVort"].tobytes()
        centre = C.c_double()
        assert gpu_lib.lbm_psi_center_2d(p.nx, p.ny, L, dp(psi), C.byref(centre)) == LBM_OK
        assert centre.value == meta["diagnostics"]["writers"]["psi"]["psi_center"]
        return
    u, v, w, T = arr("u"), arr("v"), arr("w"), arr("T")
    assert gpu_lib.lbm_tecplot_full_3d(f.encode(), p.nx, p.ny, p.nz, L, u, v, w, T) == LBM_OK
    assert open(f, "rb").read() == d["plt_write_full_fields_plt"].tobytes()
    for axis, key in enumerate(MID3):
        assert gpu_lib.lbm_tecplot_midplane_3d(f.encode(), axis, p.nx, p.ny, p.nz, L, vsc, u, v, w, T) == LBM_OK
        assert open(f, "rb").read() == d["plt_" + key].tobytes(), key
    for axis, key in enumerate(STREAM3):
        assert gpu_lib.lbm_tecplot_midplane_stream_3d(f.encode(), axis, p.nx, p.ny, p.nz, L, vsc, u, v, w) == LBM_OK
        assert open(f, "rb").read() == d["plt_" + key].tobytes(), key


@pytest.mark.parametrize("dim", [2, 3])
def test_output_binary_records(gpu_lib, tmp_path, dim):
    """output_binary (3DRB.F90:1599-1627, 2DRB.F90:1357-1389): one record per field,
    velocities scaled by velocityScaleCompare."""
    from lbmgpu import restart
    rng = np.random.default_rng(dim)
    shape = (3, 4, 5) if dim == 3 else (4, 5)
    f = {k: rng.standard_normal(shape) for k in ("u", "v", "w", "T", "rho")}
    path = str(tmp_path / "snap.bin")
    nz = shape[0] if dim == 3 else 1
    st = gpu_lib.lbm_output_binary_host(path.encode(), dim, shape[-1], shape[-2], nz, 2.5, dp(f["u"]), dp(f["v"]),
                                        dp(f["w"]), dp(f["T"]), dp(f["rho"]))
    assert st == LBM_OK
    recs = [np.frombuffer(r, dtype="<f8") for r in restart.records(path)]
    want = [2.5 * f["u"], 2.5 * f["v"]] + ([2.5 * f["w"]] if dim == 3 else []) + [f["T"], f["rho"]]
    assert len(recs) == len(want)
    for r, w in zip(recs, want):
        assert np.array_equal(r, w.ravel())
