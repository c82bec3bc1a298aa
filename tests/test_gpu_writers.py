"""Snapshot writers through a lattice handle, and the GPU fine-grid |psi| search.

The stepped state of each golden fixture is loaded into an FP64 lattice; output_Tecplot
must write the reference's files (names and bytes), output_binary the reference's records,
and calc_psi_vort_and_output (2D) the psi-vort file plus the centre value and the fine-grid
maximum of |psi| that the reference's calc_psi_absmax_fine_spline finds (fixtures computed
with 20 fine points per unit length; the search itself runs on the GPU)."""
import os

import numpy as np
import pytest

import golden_cases as gc
from lbmgpu import Lattice, restart

pytestmark = pytest.mark.gpu

FILES3 = {"fullField-": "write_full_fields_plt", "midX-": "write_midplane_x", "midY-": "write_midplane_y",
          "midZ-": "write_midplane_z", "midXpsiVort-": "write_midplane_stream_x",
          "midYpsiVort-": "write_midplane_stream_y", "midZpsiVort-": "write_midplane_stream_z"}


def loaded(name):
    meta = gc.cases()[name]
    data = gc.load(name)
    lat = Lattice(gc.params_for(meta))
    lat.initial()
    for f in gc.field_names(data):
        lat.set_state(f, data["out_" + f])
    return meta, data, lat


@pytest.mark.parametrize("name", sorted(gc.cases()))
def test_output_tecplot_files(tmp_path, name):
    meta, data, lat = loaded(name)
    prefix = str(tmp_path / "buoyancyCavity")
    lat.output_Tecplot(prefix, 1234)
    if meta["dim"] == 2:
        assert open(prefix + "-000000001234.plt", "rb").read() == data["plt_fields"].tobytes()
        got = lat.calc_psi_vort_and_output(prefix, 1234, fine_per_unit=20)
        assert open(prefix + "-psiVort-000000001234.plt", "rb").read() == data["plt_psiVort"].tobytes()
        want = meta["diagnostics"]["writers"]["psi"]
        for k in ("psi_center", "psi_abs_max", "x_at_max", "y_at_max", "psi_center_abs_fine"):
            assert got[k] == want[k], (k, got[k], want[k])
        assert got["psi_center_abs"] == abs(want["psi_center"])
    else:
        for tag, key in FILES3.items():
            path = prefix + "-" + tag + "000000001234.plt"
            assert open(path, "rb").read() == data["plt_" + key].tobytes(), tag
    lat.close()


@pytest.mark.parametrize("name", ["rb2d_periodic", "rb3d_noslip"])
def test_output_binary(tmp_path, name):
    meta, data, lat = loaded(name)
    path = str(tmp_path / "snap.bin")
    lat.output_binary(path)
    vsc = lat.constants()["velocityScaleCompare"]
    recs = [np.frombuffer(r, dtype="<f8") for r in restart.records(path)]
    names = ["u", "v"] + (["w"] if meta["dim"] == 3 else []) + ["T", "rho"]
    assert len(recs) == len(names)
    for r, k in zip(recs, names):
        want = lat.get_state(k).ravel()
        assert np.array_equal(r, vsc * want if k in ("u", "v", "w") else want), k
    lat.close()


def test_psi_search_at_the_reference_resolution():
    """The reference's own fine grid (10000 points per unit) on a 2D cavity: 2e8 spline
    evaluations; the maximum lies inside the cavity and the centre values agree."""
    from lbmgpu.abi import LBM_BCT_ADIABATIC, LBM_BCT_CONST, LBM_CELL_SIDE, rb_params
    p = rb_params(dim=2, nx=64, ny=64, Ra=1e5, noise_amp=1e-3, periodic_x=False)
    p.cell = LBM_CELL_SIDE
    p.bc_thermal[0] = LBM_BCT_CONST
    p.bc_thermal[1] = LBM_BCT_ADIABATIC
    lat = Lattice(p)
    lat.initial()
    lat.step(400)
    out = lat.calc_psi_vort_and_output(None, 0, fine_per_unit=10000)
    assert 0.0 < out["x_at_max"] < 1.0 and 0.0 < out["y_at_max"] < 1.0
    assert out["psi_abs_max"] >= out["psi_center_abs_fine"] > 0.0
    assert out["psi_center_abs"] == pytest.approx(out["psi_center_abs_fine"], rel=0.05)
    lat.close()
