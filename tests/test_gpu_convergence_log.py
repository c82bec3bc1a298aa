"""check with the reference's convergence history, on a handle (2DRB.F90:1244-1258,
3DRB.F90:1511-1526): the errors equal lbm_check's on a twin lattice, the run file and the
master file get the reference's headers, zones and records, the line is echoed to standard
output, and the case tag spells Ra, the sizes and the two switches as the reference's
write(caseTag, ...) does."""
import os

import pytest

from lbmgpu import Lattice
from lbmgpu.abi import rb_params

pytestmark = pytest.mark.gpu


def es(x):
    mant, exp = ("%.16E" % x).split("E")
    e = int(exp)
    return (mant + ("E%+03d" % e if abs(e) < 100 else "%+04d" % e)).rjust(24)


@pytest.mark.parametrize("dim", [2, 3])
def test_check_log_files_and_echo(tmp_path, capfd, dim):
    p = rb_params(dim=2, nx=32, ny=16, Ra=1e5, noise_amp=1e-3) if dim == 2 else \
        rb_params(dim=3, nx=12, ny=10, nz=8, Ra=1e6, noise_amp=1e-3)
    a, b = Lattice(p), Lattice(p)
    recs = []
    for lat in (a, b):
        lat.initial()
    for n in (7, 13):
        for lat in (a, b):
            lat.step(n)
        eu, et = a.check_log(str(tmp_path), echo=True)
        assert (eu, et) == b.check()
        recs.append((a.itc, eu, et))
    out = capfd.readouterr().out
    lines = ["%12d %s %s\n" % (itc, es(eu), es(et)) for itc, eu, et in recs]
    assert out == "".join(lines)
    tag = a.case_tag()
    if dim == 2:
        assert tag == "Ra= 1.000E+05,nx=32,ny=16,useG=T,old=F"
        run, master, zone, title = "convergence.plt", "convergence_all.plt", "conv", "Convergence comparison"
    else:
        assert tag == "Ra= 1.000E+06,nx=12,ny=10,nz=8,useG=T,old=F"
        run, master, zone, title = "convergence3D.plt", "convergence_all_3D.plt", "conv3d", "Convergence comparison 3D"
    hdr = 'VARIABLES = "itc" "errorU" "errorT"\n'
    assert open(os.path.join(str(tmp_path), run)).read() == hdr + 'ZONE T="%s", F=POINT\n' % zone + "".join(lines)
    assert open(os.path.join(str(tmp_path), master)).read() == \
        'TITLE = "%s"\n' % title + hdr + 'ZONE T="%s", F=POINT\n' % tag + "".join(lines)
    # a second run (a new handle) replaces the run file and adds a zone to the master file
    c = Lattice(p)
    c.initial()
    c.step(5)
    eu, et = c.check_log(str(tmp_path))
    line = "%12d %s %s\n" % (c.itc, es(eu), es(et))
    assert open(os.path.join(str(tmp_path), run)).read() == hdr + 'ZONE T="%s", F=POINT\n' % zone + line
    assert open(os.path.join(str(tmp_path), master)).read().endswith('ZONE T="%s", F=POINT\n' % tag + line)
    for lat in (a, b, c):
        lat.close()
