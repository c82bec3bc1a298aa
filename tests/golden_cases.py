"""Parameters and loaders for the step fixtures in tests/golden/ (generated from the
reference's own subroutines by tests/golden/make_golden.py)."""
import json
import os

import numpy as np

from lbmgpu.abi import (FIELDS, LBM_BC_NOSLIP, LBM_BC_PERIODIC, LBM_BCT_ADIABATIC, LBM_BCT_CONST, LBM_BCT_PERIODIC,
                        LBM_CELL_RB, LBM_CELL_SIDE, LbmParams)

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cases():
    with open(os.path.join(HERE, "step_cases.json")) as fh:
        return json.load(fh)


def params_for(meta):
    d = set(meta["defines"])
    p = LbmParams()
    p.dim = meta["dim"]
    p.nx, p.ny = meta["nx"], meta["ny"]
    p.nz = meta.get("nz", 1) if p.dim == 3 else 1
    p.Ra, p.Pr, p.Mach = meta["Ra"], meta["Pr"], meta["Mach"]
    p.Thot, p.Tcold = 0.5, -0.5
    p.cell = LBM_CELL_SIDE if "SideHeatedCell" in d else LBM_CELL_RB
    p.bc_flow[0] = LBM_BC_PERIODIC if "VerticalWallsPeriodicalU" in d else LBM_BC_NOSLIP
    p.bc_flow[1] = LBM_BC_NOSLIP
    p.bc_flow[2] = LBM_BC_PERIODIC if "SpanwiseWallsPeriodicalU" in d else LBM_BC_NOSLIP
    p.bc_thermal[0] = (LBM_BCT_PERIODIC if "VerticalWallsPeriodicalT" in d else
                       LBM_BCT_CONST if "VerticalWallsConstT" in d else LBM_BCT_ADIABATIC)
    p.bc_thermal[1] = LBM_BCT_CONST if "HorizontalWallsConstT" in d else LBM_BCT_ADIABATIC
    p.bc_thermal[2] = LBM_BCT_PERIODIC if "SpanwiseWallsPeriodicalT" in d else LBM_BCT_ADIABATIC
    p.use_g = 1 if "EnableUseG" in d else 0
    p.side_heated_ha = 1 if "SideHeatedHa" in d else 0
    p.Ha = meta.get("Ha", 20.0)
    p.phi_deg = meta.get("phi_deg", 0.0)
    p.legacy_thermal = 1 if "EnableLegacyThermalScheme" in d else 0
    p.precision = 0
    p.pattern = 0
    p.seed = 0
    p.noise_amp = 0.0
    return p


def load(name):
    return dict(np.load(os.path.join(HERE, "step_%s.npz" % name)))


def field_names(data):
    return sorted(k[3:] for k in data if k.startswith("in_"))


def field_id(name):
    return FIELDS[name]


def restart_names(data):
    return sorted(k[4:] for k in data if k.startswith("rst_"))
