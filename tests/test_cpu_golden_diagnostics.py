"""The oracle's post-processing diagnostics against the reference's own statements.

For every step fixture, make_golden.py ran the reference's calNuRe, RBcalc_Nu_global,
RBcalc_Nu_wall_avg, SideHeatedcalc_Nu_global, SideHeatedcalc_Nu_wall_avg and the mid-line
(2D: SideHeated/RBcalc_{u,v}mid_max) or mid-plane (3D: calc_{u,v,w}mid_max_common)
velocity maxima, transliterated from 2DRB.F90 / 3DRB.F90, on the stepped state.  The
oracle evaluates the same sums in the same order, so every number matches bit for bit.
"""
import numpy as np
import pytest

import golden_cases as gc
from lbmgpu.abi import LbmMidMax, LbmNuWall

MID = {  # fixture name -> (component, RB form)
    "SideHeatedcalc_umid_max": (0, 0), "RBcalc_umid_max": (0, 1), "SideHeatedcalc_vmid_max": (1, 0),
    "RBcalc_vmid_max": (1, 1), "calc_umid_max_common": (0, 0), "calc_vmid_max_common": (1, 0),
    "calc_wmid_max_common": (2, 0),
}


def stepped_oracle(oracle_mod, name):
    meta = gc.cases()[name]
    p = gc.params_for(meta)
    data = gc.load(name)
    o = oracle_mod.Oracle(p)
    o.initial()
    for f in gc.field_names(data):
        o.set(gc.field_id(f), data["out_" + f])
    return o, meta["diagnostics"]


@pytest.mark.parametrize("name", sorted(gc.cases()))
def test_oracle_diagnostics_match_reference(oracle_mod, name):
    o, want = stepped_oracle(oracle_mod, name)
    nu, re_, _ = o.calNuRe()
    assert (nu, re_) == (want["calNuRe"]["Nu"], want["calNuRe"]["Re"])
    assert o.RBcalc_Nu_global()[0] == want["RBcalc_Nu_global"]["Nu_global"]
    assert o.SideHeatedcalc_Nu_global()[0] == want["SideHeatedcalc_Nu_global"]["Nu_global"]
    assert o.RBcalc_Nu_wall_avg(LbmNuWall)[0].as_dict() == want["RBcalc_Nu_wall_avg"]
    assert o.SideHeatedcalc_Nu_wall_avg(LbmNuWall)[0] == want["SideHeatedcalc_Nu_wall_avg"]
    for key, (comp, rb) in MID.items():
        if key in want:
            got, st = o.mid_max(comp, rb, LbmMidMax)
            assert st == 0 and got == want[key], (key, got, want[key])


def test_mid_max_covers_every_routine():
    names = set()
    for meta in gc.cases().values():
        names |= set(meta["diagnostics"])
    assert set(MID) <= names
