"""Restart-file framing on the host (no GPU): the library's Fortran record writer and
reader against the gfortran unformatted sequential layout written out byte by byte here.

gfortran frames a record as [int32 n][n bytes][int32 n]; a record longer than 2^31 - 9
bytes is split into subrecords whose leading marker is negative when another subrecord
follows and whose trailing marker is negative when another subrecord preceded.  The
subrecord size is lowered through lbm_fortran_set_subrecord_limit so the split is
exercised on small data.  backupData's records hold f(alpha,i,j,k) with the direction
index outermost and x fastest (3DRB.F90:1661-1662, 2DRB.F90:1423-1424).
"""
import struct

import numpy as np
import pytest

from lbmgpu import restart
from lbmgpu.abi import LBM_OK


def framed(payload, limit=2147483639):
    """The bytes gfortran writes for one record."""
    n = len(payload)
    if n == 0:
        return struct.pack("<ii", 0, 0)
    out, off, first = b"", 0, True
    while off < n:
        k = min(limit, n - off)
        last = off + k == n
        out += struct.pack("<i", k if last else -k) + payload[off:off + k] + struct.pack("<i", k if first else -k)
        off += k
        first = False
    return out


@pytest.fixture
def limit(gpu_lib):
    def set_limit(n):
        assert gpu_lib.lbm_fortran_set_subrecord_limit(n) == LBM_OK
    yield set_limit
    set_limit(2147483639)


def test_single_record_bytes(gpu_lib, tmp_path):
    p = str(tmp_path / "r.bin")
    a = np.arange(10, dtype="<f8")
    restart.write_record(p, a, append=False)
    assert open(p, "rb").read() == framed(a.tobytes())


@pytest.mark.parametrize("nbytes,lim", [(80, 24), (48, 24), (8, 8), (0, 24), (1000, 7)])
def test_subrecord_bytes_and_read_back(gpu_lib, tmp_path, limit, nbytes, lim):
    p = str(tmp_path / "r.bin")
    payload = bytes((7 * k + 3) & 0xFF for k in range(nbytes))
    limit(lim)
    restart.write_record(p, np.frombuffer(payload, dtype=np.uint8), append=False)
    restart.write_record(p, np.frombuffer(b"tail-rec", dtype=np.uint8), append=True)
    assert open(p, "rb").read() == framed(payload, lim) + framed(b"tail-rec", lim)
    limit(2147483639)  # the reader follows the markers, whatever limit wrote them
    recs = list(restart.records(p))
    assert recs == [payload, b"tail-rec"]


def test_reader_rejects_bad_trailing_marker(gpu_lib, tmp_path):
    p = str(tmp_path / "bad.bin")
    open(p, "wb").write(struct.pack("<i", 16) + b"x" * 16 + struct.pack("<i", 15))
    with pytest.raises(Exception):
        list(restart.records(p))


def test_reader_reports_long_record(gpu_lib, tmp_path):
    import ctypes as C
    p = str(tmp_path / "r.bin")
    restart.write_record(p, np.arange(4, dtype="<f8"), append=False)
    buf = np.zeros(2, dtype="<f8")
    n, nxt = C.c_size_t(), C.c_uint64()
    st = gpu_lib.lbm_fortran_record_read(p.encode(), 0, buf.ctypes.data_as(C.c_void_p), buf.nbytes, C.byref(n),
                                         C.byref(nxt))
    assert st == 7 and n.value == 32 and nxt.value == 40
    assert list(buf) == [0.0, 1.0]


@pytest.mark.parametrize("dim,shape", [(2, (6, 5, 1)), (3, (4, 3, 2))])
def test_backup_layout_is_direction_major(gpu_lib, tmp_path, dim, shape):
    nx, ny, nz = shape
    q, qt = (19, 7) if dim == 3 else (9, 5)
    grid = (nz, ny, nx) if dim == 3 else (ny, nx)
    rng = np.random.default_rng(3)
    f = rng.standard_normal(grid + (q,))
    g = rng.standard_normal(grid + (qt,))
    p = str(tmp_path / restart.backup_filename(dim, 12))
    assert p.endswith("backupFile3D-12.bin" if dim == 3 else "backupFile-12.bin")
    restart.write_backup(p, f, g)
    raw = open(p, "rb").read()
    # record 1: f(alpha, i, j, k) with i fastest, alpha outermost
    n = nx * ny * nz
    vals = np.frombuffer(raw[4:4 + 8 * q * n], dtype="<f8")
    for alpha, i, j, k in [(0, 0, 0, 0), (q - 1, nx - 1, ny - 1, nz - 1), (2, 1, 2, nz - 1)]:
        want = f[k, j, i, alpha] if dim == 3 else f[j, i, alpha]
        assert vals[alpha * n + i + nx * (j + ny * k)] == want
    f2, g2 = restart.read_backup(p, dim, nx, ny, nz)
    assert np.array_equal(f2, f) and np.array_equal(g2, g)
