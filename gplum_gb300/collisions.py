"""GPLUM's collision files (collisionNNNNNN.dat, Collision0::write2File,
src/collisionA.h:122-148) from Python: the records of the last hard call and
the library's formatter.

    recs = records(lib)                 # p3t_collision_t of the last p3t_hard
    write_host(path, recs, append=True) # GPLUM's line format, no GPU
"""
import ctypes

from . import _lib


class Record(ctypes.Structure):
    _fields_ = [("time", ctypes.c_double), ("id_imp", ctypes.c_longlong), ("id_tar", ctypes.c_longlong),
                ("n_frag", ctypes.c_int), ("id_frag", ctypes.c_longlong), ("mass_imp", ctypes.c_double),
                ("mass_tar", ctypes.c_double), ("mass_frag", ctypes.c_double),
                ("pos_imp", ctypes.c_double * 3), ("pos_tar", ctypes.c_double * 3),
                ("vel_imp", ctypes.c_double * 3), ("vel_tar", ctypes.c_double * 3), ("flag", ctypes.c_int),
                ("dpos_g_rel", ctypes.c_double), ("dvel_g_rel", ctypes.c_double)]


def write_host(path, recs, append=False, lib=None):
    lib = lib or _lib.host_lib()
    arr = (Record * max(1, len(recs)))(*recs)
    _lib.check(lib.p3t_collisions_write_host(str(path).encode(), 1 if append else 0, len(recs), arr),
               "p3t_collisions_write_host")


def records(lib=None):
    """The collision records of the last hard call, in collision-list order."""
    lib = lib or _lib.host_lib()
    n = lib.p3t_collision_records(0, None)
    if n < 0:
        raise RuntimeError(f"p3t_collision_records failed with status {n}")
    arr = (Record * max(1, n))()
    lib.p3t_collision_records(n, arr)
    return list(arr)[:n]
