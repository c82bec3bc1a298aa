"""The convergence history that the reference's `check` writes (2DRB.F90:1249-1258,
1269-1343; 3DRB.F90:1522-1526, 1533-1591), through the host forms of the library's
appenders (no GPU):

* the record write(u,'(I12,1X,ES24.16,1X,ES24.16)') itc, errorU, errorT against known
  answers of the Fortran edit descriptors and against an independent Python restatement of
  ES editing on random doubles (every binade, NaN, infinities, signed zeros);
* append_convergence_tecplot: the first call of a run replaces the file with the two header
  lines and the record, later calls append (a missing file is an error, as status='old');
* append_convergence_master_tecplot: a title and variables line only when the file does not
  exist, a new zone (trailing blanks of the name trimmed) on the first call of every run.

No Fortran compiler is available to run the reference's formatted writes; the format is
pinned to the edit descriptors it names.  The handle forms (check_log, case_tag) are covered
by test_gpu_parity.py."""
import ctypes as C
import math
import os
import random

import pytest

from lbmgpu.abi import LBM_ERR_IO, LBM_OK


def es_ref(x, w, d, e=0):
    """Fortran ESw.d / ESw.dEe output of x, restated from the edit descriptor's definition."""
    if math.isnan(x):
        s = "NaN"
    elif math.isinf(x):
        s = "-Infinity" if x < 0 else "Infinity"
    else:
        mant, exp = ("%.*E" % (d, x)).split("E")
        ev = int(exp)
        digits = "%d" % abs(ev)
        sign = "-" if ev < 0 else "+"
        if e:
            if len(digits) > e:
                return "*" * w
            s = mant + "E" + sign + digits.zfill(e)
        elif len(digits) <= 2:
            s = mant + "E" + sign + digits.zfill(2)
        else:
            s = mant + sign + digits
    return "*" * w if len(s) > w else s.rjust(w)


@pytest.fixture(scope="module")
def lib(gpu_lib):
    return gpu_lib


def fmt(lib, x, w, d, e=0):
    buf = C.create_string_buffer(128)
    assert lib.lbm_format_fortran_es(C.c_double(x), w, d, e, buf, 128) == LBM_OK
    return buf.value.decode()


KNOWN = [
    (1.0, "  1.0000000000000000E+00"),
    (-1.0, " -1.0000000000000000E+00"),
    (0.0, "  0.0000000000000000E+00"),
    (-0.0, " -0.0000000000000000E+00"),
    (0.5, "  5.0000000000000000E-01"),
    (1e-100, "  1.0000000000000000-100"),
    (1e300, "  1.0000000000000001+300"),
    (5e-324, "  4.9406564584124654-324"),
    (float("nan"), "                     NaN"),
    (float("inf"), "                Infinity"),
    (-float("inf"), "               -Infinity"),
]


def test_known_answers(lib):
    for x, want in KNOWN:
        assert fmt(lib, x, 24, 16) == want, x
    assert fmt(lib, 1e7, 10, 3, 2) == " 1.000E+07"  # the caseTag's Rayleigh number
    assert fmt(lib, 2.5e-3, 10, 3, 2) == " 2.500E-03"
    assert fmt(lib, 1e100, 10, 3, 2) == "**********"  # three exponent digits do not fit E2


def test_es_against_restatement(lib):
    rng = random.Random(7)
    import struct
    for _ in range(20000):
        x = struct.unpack("<d", struct.pack("<Q", rng.getrandbits(64)))[0]
        assert fmt(lib, x, 24, 16) == es_ref(x, 24, 16), x
    for _ in range(5000):
        x = rng.uniform(-1, 1) * 10.0 ** rng.randint(-120, 120)
        assert fmt(lib, x, 10, 3, 2) == es_ref(x, 10, 3, 2), x


def line(itc, eu, et):
    return "%12d %s %s\n" % (itc, es_ref(eu, 24, 16), es_ref(et, 24, 16))


def test_record_line(lib):
    buf = C.create_string_buffer(128)
    for itc, eu, et in [(0, 0.0, 0.0), (2000, 1.5e-6, 3.25e-9), (123456789, float("nan"), 1.0)]:
        assert lib.lbm_convergence_line(itc, C.c_double(eu), C.c_double(et), buf, 128) == LBM_OK
        assert buf.value.decode() == line(itc, eu, et)


def test_run_file_replaced_then_appended(lib, tmp_path):
    for dim, zone in ((2, "conv"), (3, "conv3d")):
        path = str(tmp_path / ("convergence%d.plt" % dim))
        with open(path, "w") as f:
            f.write("stale contents of an earlier run\n")
        recs = [(2000, 1.0e-3, 2.0e-4), (4000, 5.0e-5, 1.0e-5), (6000, 7.0e-7, 3.0e-7)]
        for k, (itc, eu, et) in enumerate(recs):
            assert lib.lbm_append_convergence_tecplot_host(os.fsencode(path), 1 if k == 0 else 0, dim, itc,
                                                           C.c_double(eu), C.c_double(et)) == LBM_OK
        want = 'VARIABLES = "itc" "errorU" "errorT"\nZONE T="%s", F=POINT\n' % zone + "".join(line(*r) for r in recs)
        assert open(path).read() == want
    missing = str(tmp_path / "missing.plt")
    assert lib.lbm_append_convergence_tecplot_host(os.fsencode(missing), 0, 2, 1, C.c_double(1.0),
                                                   C.c_double(1.0)) == LBM_ERR_IO
    assert not os.path.exists(missing)


def test_master_file_zones_per_run(lib, tmp_path):
    path = str(tmp_path / "convergence_all.plt")
    runs = [("Ra= 1.000E+05,nx=256,ny=128,useG=T,old=F   ", [(2000, 1e-3, 1e-4), (4000, 1e-5, 1e-6)]),
            ("Ra= 1.000E+06,nx=256,ny=128,useG=T,old=F", [(2000, 2e-3, 2e-4)])]
    want = 'TITLE = "Convergence comparison"\nVARIABLES = "itc" "errorU" "errorT"\n'
    for zone, recs in runs:
        for k, (itc, eu, et) in enumerate(recs):
            assert lib.lbm_append_convergence_master_tecplot_host(os.fsencode(path), 1 if k == 0 else 0, 2,
                                                                  zone.encode(), itc, C.c_double(eu),
                                                                  C.c_double(et)) == LBM_OK
        want += 'ZONE T="%s", F=POINT\n' % zone.rstrip() + "".join(line(*r) for r in recs)
    assert open(path).read() == want
    path3 = str(tmp_path / "convergence_all_3D.plt")
    assert lib.lbm_append_convergence_master_tecplot_host(os.fsencode(path3), 1, 3, b"z", 1, C.c_double(0.5),
                                                          C.c_double(0.25)) == LBM_OK
    assert open(path3).read().startswith('TITLE = "Convergence comparison 3D"\n')
