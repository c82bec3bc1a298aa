"""Restart files on the GPU: backupData / reload (3DRB.F90:1638-1665, 602-623;
2DRB.F90:1402-1430, 621-637) and reconstruct_macro_from_fg (3DRB.F90:1392-1463,
2DRB.F90:1144-1200).

* The reference's reconstruction, run by the library on the f and g records of the golden
  fixtures, reproduces the fixtures' reconstructed fields (computed by executing the
  reference's own statements) bit for bit.
* A reference-format reload followed by further steps stays bitwise on the oracle's
  trajectory for the same file.
* The continuation records make a restart bit-continuous for every storage precision.
* The f and g records equal the state lbm_get_state returns, in the reference's order.
"""
import os

import numpy as np
import pytest

import golden_cases as gc
from lbmgpu import Ensemble, Lattice, LbmDiverged, LbmError, load_library, restart
from lbmgpu.abi import LBM_ERR_IO, LBM_ERR_PARAM, LBM_ERR_STATE, field_shape, rb_params

pytestmark = pytest.mark.gpu

SMALL = {2: dict(dim=2, nx=48, ny=24, Ra=1e5, Pr=0.71), 3: dict(dim=3, nx=20, ny=16, nz=12, Ra=1e6, Pr=0.71)}


def lattice(dim, precision="fp64", seed=5, **kw):
    args = dict(SMALL[dim])
    args.update(kw)
    lat = Lattice(rb_params(noise_amp=1e-3, seed=seed, precision=precision, **args))
    return lat


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp16"])
@pytest.mark.parametrize("dim", [2, 3])
def test_continuation_is_bit_continuous(tmp_path, dim, precision):
    path = str(tmp_path / restart.backup_filename(dim, 1))
    a = lattice(dim, precision)
    a.initial()
    a.step(45)  # graph chunks and single steps
    a.backupData(path, continuation=True)
    a.step(40)
    b = lattice(dim, precision, seed=99)  # a different initial field, never initialised
    assert b.reload(path, "continue") == "continue"
    assert b.itc == 45
    b.step(40)
    assert a.itc == b.itc == 85
    for name in ("f", "g", "T", "u", "v", "rho"):
        x, y = a.get_state(name), b.get_state(name)
        assert np.array_equal(x, y), (name, float(np.abs(x - y).max()))
    assert a.calNuRe() == b.calNuRe()
    a.close()
    b.close()


def test_continuation_across_subrecords(tmp_path):
    """Records split into many subrecords (limit lowered) and staged in many pieces."""
    lib = load_library()
    path = str(tmp_path / "split.bin")
    a = lattice(3, "fp32")
    a.initial()
    a.step(7)
    assert lib.lbm_fortran_set_subrecord_limit(4099) == 0
    try:
        a.backupData(path, continuation=True)
    finally:
        lib.lbm_fortran_set_subrecord_limit(2147483639)
    raw = open(path, "rb").read()
    assert int.from_bytes(raw[:4], "little", signed=True) == -4099
    b = lattice(3, "fp32")
    assert b.reload(path, "continue") == "continue"
    a.step(9)
    b.step(9)
    assert np.array_equal(a.get_state("g"), b.get_state("g"))


@pytest.mark.parametrize("name", sorted(gc.cases()))
def test_reference_reload_matches_reference_statements(tmp_path, name):
    meta = gc.cases()[name]
    p = gc.params_for(meta)
    data = gc.load(name)
    path = str(tmp_path / "fixture.bin")
    restart.write_backup(path, data["out_f"], data["out_g"])
    lat = Lattice(p)
    lat.initial()
    if not p.use_g:
        # the 2D reconstruction without EnableUseG leaves B_prev as it is
        lat.set_state("Bx_prev", data["out_Bx_prev"])
        lat.set_state("By_prev", data["out_By_prev"])
    assert lat.reload(path, "reference") == "reference"
    assert lat.itc == 0
    for f in gc.restart_names(data):
        got = lat.get_state(f)
        assert np.array_equal(got, data["rst_" + f]), (name, f, float(np.abs(got - data["rst_" + f]).max()))
    lat.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_reference_reload_continues_on_oracle_trajectory(tmp_path, oracle_mod, dim):
    path = str(tmp_path / "run.bin")
    a = lattice(dim)
    a.initial()
    a.step(30)
    a.backupData(path, continuation=False)
    assert len(list(restart.records(path))) == 2
    f, g = restart.read_backup(path, dim, a.params.nx, a.params.ny, a.params.nz)
    o = oracle_mod.Oracle(a.params)
    o.initial()
    o.set(gc.field_id("f"), f)
    o.set(gc.field_id("g"), g)
    assert not o.reconstruct_macro_from_fg()
    b = lattice(dim)
    assert b.reload(path, "auto") == "reference"
    names = ["rho", "u", "v", "T", "Bx_prev", "By_prev"] + (["w", "Bz_prev"] if dim == 3 else ["Fx", "Fy"])
    for name in names:
        assert np.array_equal(b.get_state(name), o.get(gc.field_id(name), field_shape(a.params, name))), name
    o.step(20)
    b.step(20)
    for name in ("f", "g", "T", "u"):
        x, y = b.get_state(name), o.get(gc.field_id(name), field_shape(a.params, name))
        assert np.array_equal(x, y), (name, float(np.abs(x - y).max()))
    errs_b, errs_o = b.check(), o.check()[:2]
    assert errs_b == errs_o


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp16"])
def test_backup_records_are_the_state(tmp_path, precision):
    path = str(tmp_path / "s.bin")
    a = lattice(3, precision)
    a.initial()
    a.step(33)
    a.backupData(path, continuation=False)
    f, g = restart.read_backup(path, 3, a.params.nx, a.params.ny, a.params.nz)
    assert np.array_equal(f, a.get_state("f"))
    assert np.array_equal(g, a.get_state("g"))


def test_reduced_precision_reference_reload_close_to_fp64(tmp_path):
    path = str(tmp_path / "r.bin")
    a = lattice(3)
    a.initial()
    a.step(25)
    a.backupData(path, continuation=False)
    ref = lattice(3)
    ref.reload(path, "reference")
    for precision, tol in (("fp32", 2e-6), ("fp16", 2e-3)):
        b = lattice(3, precision)
        assert b.reload(path, "auto") == "reference"
        for name in ("T", "u", "rho"):
            assert np.abs(b.get_state(name) - ref.get_state(name)).max() < tol, (precision, name)


def test_reload_errors_leave_or_drop_state_as_documented(tmp_path):
    lat = lattice(2)
    lat.initial()
    lat.step(3)
    T0 = lat.get_state("T")
    # missing file, wrong lattice size, missing continuation records: state untouched
    with pytest.raises(LbmError) as e:
        lat.reload(str(tmp_path / "none.bin"))
    assert e.value.status == LBM_ERR_IO
    other = lattice(2, nx=40)
    other.initial()
    other.backupData(str(tmp_path / "other.bin"), continuation=True)
    with pytest.raises(LbmError) as e:
        lat.reload(str(tmp_path / "other.bin"))
    assert e.value.status == LBM_ERR_IO
    lat.backupData(str(tmp_path / "ref.bin"), continuation=False)
    with pytest.raises(LbmError) as e:
        lat.reload(str(tmp_path / "ref.bin"), "continue")
    assert e.value.status == LBM_ERR_IO
    assert np.array_equal(lat.get_state("T"), T0)
    # continuation records of another precision: refused in continue mode, skipped in auto
    half = lattice(2, "fp16")
    half.initial()
    half.step(2)
    half.backupData(str(tmp_path / "half.bin"), continuation=True)
    with pytest.raises(LbmError) as e:
        lat.reload(str(tmp_path / "half.bin"), "continue")
    assert e.value.status == LBM_ERR_PARAM
    assert lat.reload(str(tmp_path / "half.bin"), "auto") == "reference"
    # an ensemble member cannot be reloaded
    m = lattice(2, "fp32")
    m.initial()
    ens = Ensemble()
    ens.add(m)
    with pytest.raises(LbmError) as e:
        m.reload(str(tmp_path / "half.bin"), "reference")
    assert e.value.status == LBM_ERR_STATE
    ens.close()
    # rho <= 0 in some cell: the reference stops; the handle is left uninitialised
    f, g = restart.read_backup(str(tmp_path / "ref.bin"), 2, lat.params.nx, lat.params.ny)
    f[3, 5, :] = 0.0
    restart.write_backup(str(tmp_path / "bad.bin"), f, g)
    with pytest.raises(LbmDiverged):
        lat.reload(str(tmp_path / "bad.bin"), "reference")
    with pytest.raises(LbmError) as e:
        lat.step(1)
    assert e.value.status == LBM_ERR_STATE
