"""Interaction lists for the soft force (host octree, see include/p3t_tree.h)."""
import ctypes
import numpy as np

from . import _lib
from .layout import SPJ_DTYPE

_I32P = ctypes.POINTER(ctypes.c_int)
_F64P = ctypes.POINTER(ctypes.c_double)
_I64P = ctypes.POINTER(ctypes.c_longlong)


def build_lists(pos, mass, r_search, theta=0.5, n_leaf_limit=8, n_group_limit=64):
    """Returns dict(n_group, i_off, i_idx, j_off, j_idx, s_off, s_idx, spj)."""
    lib = _lib.host_lib()
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    mass = np.ascontiguousarray(mass, dtype=np.float64)
    r_search = np.ascontiguousarray(r_search, dtype=np.float64)
    n = len(mass)
    t = lib.p3t_tree_build(ctypes.c_int(n), pos.ctypes.data_as(_F64P), mass.ctypes.data_as(_F64P),
                           r_search.ctypes.data_as(_F64P), ctypes.c_double(theta),
                           ctypes.c_int(n_leaf_limit), ctypes.c_int(n_group_limit))
    try:
        st = lib.p3t_tree_status(t)
        if st != 0:
            raise RuntimeError(f"p3t_tree_build failed with status {st}")
        c = np.zeros(5, np.int64)
        lib.p3t_tree_counts(t, c.ctypes.data_as(_I64P))
        ng, ni, nj, ns, nn = (int(x) for x in c)
        out = dict(n_group=ng,
                   i_off=np.zeros(ng + 1, np.int32), i_idx=np.zeros(ni, np.int32),
                   j_off=np.zeros(ng + 1, np.int32), j_idx=np.zeros(nj, np.int32),
                   s_off=np.zeros(ng + 1, np.int32), s_idx=np.zeros(ns, np.int32),
                   spj=np.zeros(nn, SPJ_DTYPE))
        lib.p3t_tree_export(t, *(out[k].ctypes.data_as(_I32P) for k in
                                 ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx")),
                            out["spj"].ctypes.data_as(_F64P))
        return out
    finally:
        lib.p3t_tree_free(t)
