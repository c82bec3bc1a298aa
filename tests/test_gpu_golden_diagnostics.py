"""The library's post-processing diagnostics against the reference's own statements.

The state after a golden step fixture is loaded into an FP64 lattice; calNuRe, the RB and
side-heated Nu_global / Nu_wall_avg and the mid-line / mid-plane velocity maxima must give
the numbers the reference's transliterated subroutines gave.  Wall profiles, fits and
mid-plane maxima are evaluated in the reference's order (bitwise); volume and plane sums
are parallel reductions on the GPU, so those agree to a few ulps of the sum
(relative 1e-12).
"""
import pytest

import golden_cases as gc
from lbmgpu import Lattice

pytestmark = pytest.mark.gpu
RTOL = 1e-12

MID = {
    2: {"SideHeatedcalc_umid_max": "SideHeatedcalc_umid_max", "RBcalc_umid_max": "RBcalc_umid_max",
        "SideHeatedcalc_vmid_max": "SideHeatedcalc_vmid_max", "RBcalc_vmid_max": "RBcalc_vmid_max"},
    3: {"calc_umid_max_common": ("SideHeatedcalc_umid_max", "RBcalc_umid_max"),
        "calc_vmid_max_common": ("SideHeatedcalc_vmid_max", "RBcalc_vmid_max"),
        "calc_wmid_max_common": ("SideHeatedcalc_wmid_max", "RBcalc_wmid_max")},
}


def close(a, b):
    return a == pytest.approx(b, rel=RTOL, abs=1e-12)


@pytest.mark.parametrize("name", sorted(gc.cases()))
def test_library_diagnostics_match_reference(name):
    meta = gc.cases()[name]
    p = gc.params_for(meta)
    data = gc.load(name)
    want = meta["diagnostics"]
    lat = Lattice(p)
    lat.initial()
    for f in gc.field_names(data):
        lat.set_state(f, data["out_" + f])
    nu, re_ = lat.calNuRe()
    assert close(nu, want["calNuRe"]["Nu"]) and close(re_, want["calNuRe"]["Re"])
    assert close(lat.RBcalc_Nu_global(), want["RBcalc_Nu_global"]["Nu_global"])
    assert close(lat.SideHeatedcalc_Nu_global(), want["SideHeatedcalc_Nu_global"]["Nu_global"])
    for fn in ("RBcalc_Nu_wall_avg", "SideHeatedcalc_Nu_wall_avg"):
        got = getattr(lat, fn)()
        for k, v in want[fn].items():
            assert close(got[k], v), (fn, k, got[k], v)
    for key, entry in MID[meta["dim"]].items():
        for fn in ((entry,) if isinstance(entry, str) else entry):
            got = getattr(lat, fn)()
            assert got == want[key], (fn, got, want[key])
    lat.close()


def test_reduced_precision_side_heated_close():
    """FP32 storage: the side-heated diagnostics of a side-heated cavity stay close to FP64."""
    from lbmgpu.abi import LBM_BCT_ADIABATIC, LBM_BCT_CONST, LBM_CELL_SIDE, rb_params
    out = {}
    for prec in ("fp64", "fp32"):
        p = rb_params(dim=3, n=24, Ra=1e5, noise_amp=1e-3, precision=prec)
        p.cell = LBM_CELL_SIDE
        p.bc_thermal[0] = LBM_BCT_CONST
        p.bc_thermal[1] = LBM_BCT_ADIABATIC
        lat = Lattice(p)
        lat.initial()
        lat.step(300)
        out[prec] = (lat.SideHeatedcalc_Nu_global(), lat.SideHeatedcalc_Nu_wall_avg(), lat.SideHeatedcalc_wmid_max())
        lat.close()
    assert out["fp32"][0] == pytest.approx(out["fp64"][0], rel=1e-4)
    assert out["fp32"][1]["Nu_hot"] == pytest.approx(out["fp64"][1]["Nu_hot"], rel=1e-4)
    assert out["fp32"][2]["value"] == pytest.approx(out["fp64"][2]["value"], rel=1e-3)
