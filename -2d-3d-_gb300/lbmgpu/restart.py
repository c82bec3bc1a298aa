"""Restart files in the reference's format, on the host.

backupData (3DRB.F90:1638-1665, 2DRB.F90:1402-1430) writes two Fortran unformatted
sequential records, f(alpha,i,j,k) then g(alpha,i,j,k) as FP64 with the direction index
outermost and x fastest; loadInitField = 1 reads them back (3DRB.F90:602-623).  These
helpers read and write such files through liblbmgpu.so's record functions (host code, no
GPU needed), for post-processing and for handing files to and from the Fortran program.
"""
import ctypes as C
import os

import numpy as np

from . import LbmError, load_library
from .abi import LBM_OK


def backup_filename(dim, number):
    """The reference's file name for backup number `number`: backupFile-<n>.bin (2D,
    2DRB.F90:1420) or backupFile3D-<n>.bin (3D, 3DRB.F90:1656)."""
    return ("backupFile3D-%d.bin" if dim == 3 else "backupFile-%d.bin") % int(number)


def write_record(path, data, append=True):
    a = np.ascontiguousarray(data)
    st = load_library().lbm_fortran_record_write(os.fsencode(path), 1 if append else 0,
                                                  a.ctypes.data_as(C.c_void_p), a.nbytes)
    if st != LBM_OK:
        raise LbmError(st, "cannot write a record to %s" % path)


def records(path):
    """Yield every record of the file as raw bytes."""
    lib = load_library()
    size = os.path.getsize(path)
    off = 0
    while off < size:
        n, nxt = C.c_size_t(), C.c_uint64()
        st = lib.lbm_fortran_record_read(os.fsencode(path), off, None, 0, C.byref(n), C.byref(nxt))
        if st not in (LBM_OK, 7):
            raise LbmError(st, "malformed record at byte %d of %s" % (off, path))
        buf = np.empty(n.value, dtype=np.uint8)
        st = lib.lbm_fortran_record_read(os.fsencode(path), off, buf.ctypes.data_as(C.c_void_p), buf.nbytes,
                                         C.byref(n), C.byref(nxt))
        if st != LBM_OK:
            raise LbmError(st, "malformed record at byte %d of %s" % (off, path))
        yield buf.tobytes()
        off = nxt.value


def _grid(dim, nx, ny, nz):
    return (nz, ny, nx) if dim == 3 else (ny, nx)


def read_backup(path, dim, nx, ny, nz=1):
    """(f, g) of a restart file in lbm_get_state's layout: [(k,) j, i, alpha]."""
    it = records(path)
    q, qt = (19, 7) if dim == 3 else (9, 5)
    grid = _grid(dim, nx, ny, nz)
    out = []
    for qq in (q, qt):
        raw = np.frombuffer(next(it), dtype="<f8")
        if raw.size != qq * int(np.prod(grid)):
            raise ValueError("record holds %d values, expected %d" % (raw.size, qq * int(np.prod(grid))))
        out.append(np.ascontiguousarray(np.moveaxis(raw.reshape((qq,) + grid), 0, -1)))
    return tuple(out)


def write_backup(path, f, g):
    """Write f and g (lbm_get_state layout, direction last) as the reference's two records."""
    for k, a in enumerate((f, g)):
        rec = np.ascontiguousarray(np.moveaxis(np.asarray(a, dtype="<f8"), -1, 0))
        write_record(path, rec, append=k > 0)
