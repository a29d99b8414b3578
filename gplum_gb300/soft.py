"""Soft force on the GPU through the C ABI (include/gplum_p3t.h).

Python mirror of GPLUM's soft-force operator surface:

* :func:`calc_force_epep` / :func:`calc_force_epsp` -- the functor calls of
  ``calcForceEPEPWithSearch`` / ``calcForceEPSP`` (src/gravity_kernel.hpp),
  same arguments, accumulate-into ``ForceGrav`` records;
* :class:`MultiWalk` -- the FDPS multiwalk dispatch/retrieve pair;
* :class:`SoftForce` -- the device-resident form (particles and lists stay in
  HBM between calls).

Every call goes to the CUDA library; there is no host fallback and a missing
GPU raises.
"""
import ctypes

import numpy as np

from . import _lib
from .layout import EPI_DTYPE, EPJ_DTYPE, FORCE_DTYPE, SPJ_DTYPE

VP = ctypes.c_void_p


def _vp(a):
    return a.ctypes.data_as(VP)


def _lib_checked():
    lib = _lib.host_lib()
    st = lib.p3t_init(0)
    if st != 0:
        raise RuntimeError(f"gplum_p3t: no usable CUDA device (status {st})")
    return lib


def configure(params, precision=0, trace_mode=0, cand_cap=64):
    lib = _lib_checked()
    v = np.ascontiguousarray(params.vector())
    _lib.check(lib.p3t_set_params(_vp(v)), "p3t_set_params")
    _lib.check(lib.p3t_set_options(precision, trace_mode, cand_cap), "p3t_set_options")
    return lib


def epj_records(pos, vel, mass, r_out, r_search, ids=None, acc_d=None):
    """EPJGrav records for particles 0..n-1 (id_local = index, rank 0)."""
    n = len(mass)
    e = np.zeros(n, EPJ_DTYPE)
    e["id_local"] = np.arange(n)
    e["pos"] = pos
    e["r_out"] = r_out
    e["r_search"] = r_search
    e["id"] = np.arange(n) if ids is None else ids
    e["mass"] = mass
    e["vel"] = vel
    if acc_d is not None:
        e["acc_d"] = acc_d
    return e


def epi_records(epj):
    e = np.zeros(len(epj), EPI_DTYPE)
    for k in EPI_DTYPE.names:
        e[k] = epj[k]
    return e


def calc_force_epep(epi, epj, force):
    """calcForceEPEPWithSearch()(epi, ni, epj, nj, force): accumulates into force."""
    lib = _lib_checked()
    epi = np.ascontiguousarray(epi, EPI_DTYPE)
    epj = np.ascontiguousarray(epj, EPJ_DTYPE)
    assert force.dtype == FORCE_DTYPE and force.flags.c_contiguous
    _lib.check(lib.p3t_epep(_vp(epi), len(epi), _vp(epj), len(epj), _vp(force)), "p3t_epep")
    return force


def calc_force_epsp(epi, spj, force):
    """calcForceEPSP()(epi, ni, spj, nj, force): accumulates into force."""
    lib = _lib_checked()
    epi = np.ascontiguousarray(epi, EPI_DTYPE)
    spj = np.ascontiguousarray(spj, SPJ_DTYPE)
    assert force.dtype == FORCE_DTYPE and force.flags.c_contiguous
    _lib.check(lib.p3t_epsp(_vp(epi), len(epi), _vp(spj), len(spj), _vp(force)), "p3t_epsp")
    return force


def _ptr_array(arrs):
    return (VP * len(arrs))(*[a.ctypes.data for a in arrs])


def _int_array(vals):
    return np.ascontiguousarray(np.asarray(vals, dtype=np.int32))


class MultiWalk:
    """FDPS calcForceAllAndWriteBackMultiWalk dispatch/retrieve."""

    def __init__(self):
        self.lib = _lib_checked()
        self._keep = {}

    def dispatch(self, tag, epis, epjs, spjs):
        epis = [np.ascontiguousarray(a, EPI_DTYPE) for a in epis]
        epjs = [np.ascontiguousarray(a, EPJ_DTYPE) for a in epjs]
        spjs = [np.ascontiguousarray(a, SPJ_DTYPE) for a in spjs]
        ne, nj, ns = (_int_array([len(a) for a in x]) for x in (epis, epjs, spjs))
        self._keep[tag] = (epis, epjs, spjs, ne)
        st = self.lib.p3t_soft_dispatch(tag, len(epis), _ptr_array(epis), _vp(ne), _ptr_array(epjs), _vp(nj),
                                        _ptr_array(spjs), _vp(ns))
        _lib.check(st, "p3t_soft_dispatch")

    def dispatch_index(self, tag, epis, id_epj, id_spj, epj, spj, send_flag=True):
        epis = [np.ascontiguousarray(a, EPI_DTYPE) for a in epis]
        id_epj = [np.ascontiguousarray(a, np.int32) for a in id_epj]
        id_spj = [np.ascontiguousarray(a, np.int32) for a in id_spj]
        epj = np.ascontiguousarray(epj, EPJ_DTYPE)
        spj = np.ascontiguousarray(spj, SPJ_DTYPE)
        ne, nj, ns = (_int_array([len(a) for a in x]) for x in (epis, id_epj, id_spj))
        self._keep[tag] = (epis, id_epj, id_spj, ne, epj, spj)
        st = self.lib.p3t_soft_dispatch_index(tag, len(epis), _ptr_array(epis), _vp(ne), _ptr_array(id_epj),
                                              _vp(nj), _ptr_array(id_spj), _vp(ns), _vp(epj), len(epj),
                                              _vp(spj), len(spj), 1 if send_flag else 0)
        _lib.check(st, "p3t_soft_dispatch_index")

    def retrieve(self, tag):
        epis, ne = self._keep[tag][0], self._keep[tag][3]
        forces = [np.zeros(len(a), FORCE_DTYPE) for a in epis]
        st = self.lib.p3t_soft_retrieve(tag, len(epis), _vp(ne), _ptr_array(forces))
        _lib.check(st, "p3t_soft_retrieve")
        del self._keep[tag]
        return forces


class SoftForce:
    """Device-resident soft force: upload once, run many times."""

    def __init__(self, params, precision=0, trace_mode=0, cand_cap=64):
        self.lib = configure(params, precision, trace_mode, cand_cap)
        self.n = 0

    def upload_particles(self, epj):
        epj = np.ascontiguousarray(epj, EPJ_DTYPE)
        _lib.check(self.lib.p3t_upload_particles(len(epj), _vp(epj)), "p3t_upload_particles")
        self.n = len(epj)

    def upload_lists(self, L):
        _lib.check(self.lib.p3t_upload_lists(L["n_group"], _vp(L["i_off"]), _vp(L["i_idx"]), _vp(L["j_off"]),
                                             _vp(L["j_idx"]), _vp(L["s_off"]), _vp(L["s_idx"]),
                                             _vp(L["spj"]), len(L["spj"])), "p3t_upload_lists")

    def run(self, emit_candidates=False):
        _lib.check(self.lib.p3t_soft_run(1 if emit_candidates else 0), "p3t_soft_run")

    def download(self, out=None):
        if out is None:
            out = np.zeros(self.n, FORCE_DTYPE)
        st = self.lib.p3t_download_forces(_vp(out), self.n)
        _lib.check(st, "p3t_download_forces")
        return out

    def stream(self):
        return self.lib.p3t_stream()

    def synchronize(self):
        _lib.check(self.lib.p3t_synchronize(), "p3t_synchronize")


def soft_force_host(params, epj, L, precision=0, trace_mode=0, out=None):
    """One call, host buffers in and out (p3t_soft_force_host)."""
    lib = configure(params, precision, trace_mode)
    epj = np.ascontiguousarray(epj, EPJ_DTYPE)
    if out is None:
        out = np.zeros(len(epj), FORCE_DTYPE)
    st = lib.p3t_soft_force_host(len(epj), _vp(epj), L["n_group"], _vp(L["i_off"]), _vp(L["i_idx"]),
                                 _vp(L["j_off"]), _vp(L["j_idx"]), _vp(L["s_off"]), _vp(L["s_idx"]),
                                 _vp(L["spj"]), len(L["spj"]), _vp(out))
    _lib.check(st, "p3t_soft_force_host")
    return out
