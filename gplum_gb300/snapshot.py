"""GPLUM's snapshot files from Python: snapNNNNNN.dat (ASCII) and
snap_tmp.dat (binary restart), through the library's writers and readers
(gplum_gb300/csrc/snapshot_io.cpp, snapshot.cu).

    hdr = Header(time=t, id_next=g.id_next(), e_init=e0, e_now=e1)
    write_host(path, binary, hdr, bodies)      # host arrays -> file (no GPU)
    hdr, bodies = read_host(path, binary)      # file -> host arrays (no GPU)
    GpuSystem.write_snapshot / read_snapshot   # device state <-> file

Energies are GPLUM's Energy fields in order (etot, ekin, ephi_sun,
ephi_planet, ephi, ephi_d, edisp), src/energy.h:3-11.
"""
import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib

ENERGY_FIELDS = ("etot", "ekin", "ephi_sun", "ephi_planet", "ephi", "ephi_d", "edisp")


class _Header(ctypes.Structure):
    _fields_ = [("n_body", ctypes.c_int), ("id_next", ctypes.c_int), ("time", ctypes.c_double),
                ("e_init", ctypes.c_double * 7), ("e_now", ctypes.c_double * 7)]


_PTR_FIELDS = [("id", ctypes.c_longlong, 1), ("mass", ctypes.c_double, 1), ("r_planet", ctypes.c_double, 1),
               ("f", ctypes.c_double, 1), ("pos", ctypes.c_double, 3), ("vel", ctypes.c_double, 3),
               ("acc", ctypes.c_double, 3), ("acc_d", ctypes.c_double, 3), ("jerk_d", ctypes.c_double, 3),
               ("acc_s", ctypes.c_double, 3), ("jerk_s", ctypes.c_double, 3), ("phi", ctypes.c_double, 1),
               ("phi_d", ctypes.c_double, 1), ("phi_s", ctypes.c_double, 1), ("r_out", ctypes.c_double, 1),
               ("r_search", ctypes.c_double, 1), ("r_out_inv", ctypes.c_double, 1), ("v_disp", ctypes.c_double, 1),
               ("time", ctypes.c_double, 1), ("dt", ctypes.c_double, 1), ("acc0", ctypes.c_double, 1),
               ("id_cluster", ctypes.c_longlong, 1), ("number", ctypes.c_int, 1), ("rank", ctypes.c_int, 1),
               ("id_max", ctypes.c_int, 1), ("id_min", ctypes.c_int, 1), ("n_cluster", ctypes.c_int, 1),
               ("dead", ctypes.c_int, 1), ("merged", ctypes.c_int, 1)]
ASCII_FIELDS = ("id", "mass", "r_planet", "f", "pos", "vel", "number")
_NP = {ctypes.c_longlong: np.int64, ctypes.c_double: np.float64, ctypes.c_int: np.int32}


class _Bodies(ctypes.Structure):
    _fields_ = [(name, ctypes.POINTER(t)) for name, t, _ in _PTR_FIELDS]


@dataclass
class Header:
    time: float = 0.0
    id_next: int = 0
    n_body: int = 0
    e_init: np.ndarray = field(default_factory=lambda: np.zeros(7))
    e_now: np.ndarray = field(default_factory=lambda: np.zeros(7))

    def _c(self):
        h = _Header()
        h.n_body, h.id_next, h.time = int(self.n_body), int(self.id_next), float(self.time)
        for k in range(7):
            h.e_init[k] = float(self.e_init[k])
            h.e_now[k] = float(self.e_now[k])
        return h

    @staticmethod
    def _from(h):
        return Header(time=h.time, id_next=h.id_next, n_body=h.n_body, e_init=np.array(h.e_init[:]),
                      e_now=np.array(h.e_now[:]))


def energy7(e5, edisp=0.0):
    """GPLUM's Energy (7 fields) from p3t_energy's {etot, ekin, ephi_sun, ephi,
    ephi_d} and the dissipated energy."""
    etot, ekin, ephi_sun, ephi, ephi_d = (float(x) for x in e5[:5])
    return np.array([etot, ekin, ephi_sun, ephi + ephi_d, ephi, ephi_d, edisp])


def _bodies(arrays):
    b = _Bodies()
    keep = []
    for name, t, w in _PTR_FIELDS:
        a = arrays.get(name)
        if a is None:
            continue
        a = np.ascontiguousarray(a, dtype=_NP[t])
        keep.append(a)
        setattr(b, name, a.ctypes.data_as(ctypes.POINTER(t)))
    return b, keep


def write_host(path, binary, header, arrays, lib=None):
    """Writes `arrays` (dict of host arrays: id, mass, r_planet, f, pos, vel,
    number, ... ) in GPLUM's format; no GPU."""
    lib = lib or _lib.host_lib()
    b, keep = _bodies(arrays)
    h = header._c()
    n = len(arrays["id"])
    _lib.check(lib.p3t_snapshot_write_host(str(path).encode(), int(binary), ctypes.byref(h), n, ctypes.byref(b)),
               "p3t_snapshot_write_host")


def read_host(path, binary, lib=None):
    """(Header, dict of host arrays) of a GPLUM snapshot file; no GPU."""
    lib = lib or _lib.host_lib()
    h = _Header()
    n = lib.p3t_snapshot_read_host(str(path).encode(), int(binary), ctypes.byref(h), 0, None)
    if n < 0:
        raise RuntimeError(f"p3t_snapshot_read_host failed with status {n}")
    names = [f for f, _, _ in _PTR_FIELDS] if binary else list(ASCII_FIELDS)
    arrays = {}
    for name, t, w in _PTR_FIELDS:
        if name in names:
            arrays[name] = np.zeros((n, 3) if w == 3 else n, dtype=_NP[t])
    b, keep = _bodies(arrays)
    r = lib.p3t_snapshot_read_host(str(path).encode(), int(binary), ctypes.byref(h), max(n, 1), ctypes.byref(b))
    if r < 0:
        raise RuntimeError(f"p3t_snapshot_read_host failed with status {r}")
    return Header._from(h), arrays
