"""Known-answer tests of the CPU oracle (no GPU needed).

The reference ships no tests or golden vectors, so the oracle is pinned by:
  * its transform matrices against the reference's own statements of them
    (tests/golden/reference_matrices.json, generated from the Fortran source text);
  * exact invariants of the scheme: M Minv = I, mass conservation with no-slip walls,
    a fluid at rest with uniform T = Tref staying exactly at rest, equilibrium being a
    fixed point of the collision.
"""
import json
import os

import numpy as np
import pytest

from lbmgpu.abi import LbmConstants, LbmNuWall, field_shape, rb_params, LBM_BCT_ADIABATIC, FIELDS

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("q", [9, 5, 19, 7])
def test_transforms_invert(oracle_mod, q):
    M, Minv = oracle_mod.transform_matrices(q)
    assert np.abs(M @ Minv - np.eye(q)).max() < 1e-14
    assert np.abs(Minv @ M - np.eye(q)).max() < 1e-14


@pytest.mark.parametrize("q", [9, 5, 19, 7])
def test_transforms_match_reference_text(oracle_mod, q):
    with open(os.path.join(GOLDEN, "reference_matrices.json")) as fh:
        gold = json.load(fh)
    M, Minv = oracle_mod.transform_matrices(q)
    ref = gold["D2Q9" if q == 9 else "D2Q5" if q == 5 else "D3Q19" if q == 19 else "D3Q7"]
    np.testing.assert_array_equal(M, np.array(ref["M"]))
    np.testing.assert_allclose(Minv, np.array(ref["Minv"]), rtol=0, atol=1e-16)


def test_d2q9_matrix_matches_independent_statement():
    """ChaiPRE2020.F90:263-276 states the D2Q9/D2Q5 matrices as rows; 2DRB.F90 expands
    them by hand.  The two statements of the reference must agree."""
    with open(os.path.join(GOLDEN, "reference_matrices.json")) as fh:
        gold = json.load(fh)
    np.testing.assert_array_equal(np.array(gold["D2Q9"]["M"]), np.array(gold["Chai_Mflow"]))
    np.testing.assert_array_equal(np.array(gold["D2Q5"]["M"]), np.array(gold["Chai_Mtemp"]))
    np.testing.assert_array_equal(np.array(gold["D3Q7"]["M"]), np.array(gold["guide_N"]))


def _run(oracle_mod, p, n):
    o = oracle_mod.Oracle(p)
    o.initial()
    o.step(n)
    return o


def test_mass_conserved_noslip_3d(oracle_mod):
    p = rb_params(dim=3, n=10, Ra=1e5, noise_amp=1e-3)
    o = oracle_mod.Oracle(p)
    o.initial()
    f0 = o.get(FIELDS["f"], field_shape(p, "f")).sum()
    o.step(50)
    f1 = o.get(FIELDS["f"], field_shape(p, "f")).sum()
    assert abs(f1 - f0) / f0 < 1e-13


def test_rest_state_stays_at_rest(oracle_mod):
    """No heated wall and T = Tref: the fluid stays at rest for 20 steps."""
    for dim in (2, 3):
        p = rb_params(dim=dim, n=8, ny=8, Ra=1e6, noise_amp=0.0)
        p.bc_thermal[1] = LBM_BCT_ADIABATIC  # no heated wall: T = 0 = Tref everywhere
        o = _run(oracle_mod, p, 20)
        f = o.get(FIELDS["f"], field_shape(p, "f"))
        w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4) if dim == 2 else \
            np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
        # the moment-space round trip rounds, so rest is kept to a few ulps, not bitwise
        assert np.abs(f - w).max() < 2e-15
        assert np.abs(o.get(FIELDS["u"], field_shape(p, "u"))).max() < 1e-15


def test_equilibrium_is_fixed_point_of_collision(oracle_mod):
    """With T = Tref (no buoyancy), f = feq(rho,u) must come out of the MRT collision
    unchanged up to rounding (m - meq = 0 for every relaxed moment)."""
    for dim in (2, 3):
        p = rb_params(dim=dim, n=6, ny=6, Ra=1e5, noise_amp=0.0)
        p.bc_thermal[1] = LBM_BCT_ADIABATIC
        o = oracle_mod.Oracle(p)
        o.initial()
        rng = np.random.default_rng(7)
        shp = field_shape(p, "rho")
        rho = 1.0 + 0.01 * rng.standard_normal(shp)
        u = 0.05 * rng.standard_normal(shp)
        v = 0.05 * rng.standard_normal(shp)
        w = 0.05 * rng.standard_normal(shp) if dim == 3 else np.zeros(shp)
        if dim == 2:
            ex = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1]); ey = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1]); ez = 0 * ex
            wt = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
        else:
            ex = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
            ey = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1])
            ez = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])
            wt = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
        eu = u[..., None] * ex + v[..., None] * ey + w[..., None] * ez
        usq = (u * u + v * v + w * w)[..., None]
        feq = rho[..., None] * wt * (1 + 3 * eu + 4.5 * eu * eu - 1.5 * usq)
        o.set(FIELDS["f"], feq)
        o.set(FIELDS["rho"], rho)
        o.set(FIELDS["u"], u)
        o.set(FIELDS["v"], v)
        if dim == 3:
            o.set(FIELDS["w"], w)
        o.collision()
        fpost = o.get(FIELDS["f_post"], field_shape(p, "f_post"))
        # 2D D2Q9 meq has no u^3 terms: feq is its exact fixed point only to O(u^3)
        tol = 1e-13 if dim == 3 else 2e-5
        assert np.abs(fpost - feq).max() < tol


def test_constants_rb2d_256x128(oracle_mod):
    """The 2D reference case (256x128, Ra 1e5, Pr 0.71, U 0.1): nu = U H sqrt(Pr/Ra)."""
    p = rb_params(dim=2, ny=128, Ra=1e5, Pr=0.71, U=0.1)
    o = oracle_mod.Oracle(p)
    c = o.constants(LbmConstants)
    nu = 0.1 * 128 * np.sqrt(0.71 / 1e5)
    assert c.viscosity == pytest.approx(nu, rel=1e-14)
    assert c.tauf == pytest.approx(0.5 + 3 * nu, rel=1e-14)
    assert c.diffusivity == pytest.approx(nu / 0.71, rel=1e-14)
    assert c.gBeta == pytest.approx(0.1 ** 2 / 128, rel=1e-13)  # U^2/(dT H)
    assert c.taug == pytest.approx(0.5 + 3 * nu / 0.71, rel=1e-14)
    assert round(c.tauf, 4) == 0.6023 and round(c.taug, 4) == 0.6441


def test_nu_conduction_state_is_one(oracle_mod):
    """A pure conduction profile (no noise, Ra below onset) has Nu = 1 to discretisation
    accuracy at t = 0 on every definition the reference uses."""
    p = rb_params(dim=3, n=12, Ra=1e5, noise_amp=0.0)
    o = oracle_mod.Oracle(p)
    o.initial()
    o.macroT()
    nu, re, st = o.calNuRe()
    assert st == 0 and nu == pytest.approx(1.0, abs=1e-12) and re == 0.0
    g, st = o.RBcalc_Nu_global()
    assert g == pytest.approx(1.0, rel=1e-3)
    wall, st = o.RBcalc_Nu_wall_avg(LbmNuWall)
    assert wall.Nu_hot == pytest.approx(1.0, rel=1e-9) and wall.Nu_cold == pytest.approx(1.0, rel=1e-9)
