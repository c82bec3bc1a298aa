"""The oracle against the reference's own subroutines.

tests/golden/step_*.npz hold module states before and after a few steps computed by
executing the reference's collision, streaming, bounceback, macro, collisionT,
streamingT, bouncebackT and macroT statements (transliterated mechanically from
2DRB.F90 / 3DRB.F90 by tests/golden/make_golden.py) on perturbed inputs, for four switch
sets: 2D RB x-periodic, 3D RB no-slip, 3D side-heated (the file's default switches) and
3D RB x/z-periodic with the legacy thermal scheme.  The oracle must reproduce every field
bit for bit.
"""
import numpy as np
import pytest

import golden_cases as gc
from lbmgpu.abi import field_shape


@pytest.mark.parametrize("name", sorted(gc.cases()))
def test_oracle_reproduces_reference_steps(oracle_mod, name):
    meta = gc.cases()[name]
    p = gc.params_for(meta)
    data = gc.load(name)
    o = oracle_mod.Oracle(p)
    o.initial()
    for f in gc.field_names(data):
        o.set(gc.field_id(f), data["in_" + f])
    o.step(meta["steps"])
    for f in gc.field_names(data):
        got = o.get(gc.field_id(f), field_shape(p, f))
        want = data["out_" + f]
        assert np.array_equal(got, want), (name, f, float(np.abs(got - want).max()))


def test_fixture_constants_match_derivation(oracle_mod):
    from lbmgpu.abi import LbmConstants
    for name, meta in gc.cases().items():
        c = oracle_mod.Oracle(gc.params_for(meta)).constants(LbmConstants)
        for k, v in meta["constants"].items():
            assert getattr(c, k) == v, (name, k, getattr(c, k), v)


@pytest.mark.parametrize("name", sorted(gc.cases()))
def test_oracle_reproduces_reference_restart(oracle_mod, name):
    """Restart: f and g after the steps, then macroT + reconstruct_macro_from_fg
    (2DRB.F90:1144-1200, 3DRB.F90:1392-1463) executed from the reference's statements."""
    meta = gc.cases()[name]
    p = gc.params_for(meta)
    data = gc.load(name)
    o = oracle_mod.Oracle(p)
    o.initial()
    for f in gc.field_names(data):
        o.set(gc.field_id(f), data["in_" + f])
    o.step(meta["steps"])
    assert not o.reconstruct_macro_from_fg()
    for f in gc.restart_names(data):
        got = o.get(gc.field_id(f), field_shape(p, f))
        want = data["rst_" + f]
        assert np.array_equal(got, want), (name, f, float(np.abs(got - want).max()))


def test_oracle_restart_flags_nonpositive_rho(oracle_mod):
    name = "rb2d_periodic"
    meta = gc.cases()[name]
    p = gc.params_for(meta)
    data = gc.load(name)
    o = oracle_mod.Oracle(p)
    o.initial()
    f = data["in_f"].copy()
    f[2, 3, :] = 0.0  # one cell with rho = 0
    o.set(gc.field_id("f"), f)
    o.set(gc.field_id("g"), data["in_g"])
    assert o.reconstruct_macro_from_fg()
