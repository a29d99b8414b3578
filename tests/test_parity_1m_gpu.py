"""Parity at the sizes the benchmark runs: the 1,048,576-body disks.

* Correction + neighbour search, cluster formation and the hard part of one
  tree step on the batched-hard-part disk, device and oracle started from
  identical inputs at each phase (the device state handed to the oracle as
  GPLUM FPGrav records): the neighbour pair list (NeighborList::pair_list,
  src/neighbor.h:635-670), neighbour counts, id_cluster and the cluster
  memberships (src/neighbor.h:800-839, src/hard.h:321-438) and the collision
  pairs (src/hermite.h:98-196) bit-exact; positions and velocities after the
  hard part within 1e-13 relative; every cluster member's block step equal,
  the few differing ones on isolated bodies only (their Kepler drift,
  src/kepler.h, calls sin/cos/atan2, which the CUDA math library and glibc
  may round differently in the last bit).
* The soft force on the 1M soft-force disk's lists: neighbour counts, rank
  sums, id_min/id_max bit-exact against GPLUM's FP32 functors
  (src/gravity_kernel.hpp:25-238); forces against the FP64 restatement with
  the mixed kernel's error below GPLUM's FP32 functor's at the median and
  the 99th percentile.
"""
import ctypes
import os

import numpy as np
import pytest

from gplum_gb300 import autotune, scheduler, soft
from gplum_gb300.disk import P3TParams, disk_1m_hard, disk_1m_soft
from gplum_gb300.layout import FORCE_DTYPE, cleared_forces
from gplum_gb300.p3t import GpuSystem
from oracle import harness as H
from tests.common import rel_err

pytestmark = pytest.mark.gpu
N = 1048576
VP = ctypes.c_void_p


def _to_oracle(orc, g):
    rec = g.get_fpgrav()
    orc.lib.orc_put_fpgrav(ctypes.c_int(len(rec)), rec.ctypes.data_as(VP), ctypes.c_longlong(g.id_next()))


def _clusters_from(idc, num):
    """Cluster memberships as a set of frozensets of body indices."""
    sel = np.nonzero(num > 0)[0]
    order = np.argsort(idc[sel], kind="stable")
    s = sel[order]
    keys = idc[s]
    cut = np.nonzero(np.diff(keys))[0] + 1
    return {frozenset(x.tolist()) for x in np.split(s, cut)}


def test_step_phases_match_the_oracle_at_1m_bodies(gpu):
    P = P3TParams(n_group_limit=256)
    g = GpuSystem(P)
    autotune.load(g.lib)
    scheduler.load(lib=g.lib)
    g.lib.p3t_set_hard_mode(0)
    g.lib.p3t_set_schedule(1)
    g.load(disk_1m_hard(N))
    g.set_r_planet()
    g.startup()
    g.kick()
    # soft force on the device lists, then the correction from identical inputs
    g.tree_soft()
    f = np.zeros(g.n, FORCE_DTYPE)
    assert g.lib.p3t_download_forces(f.ctypes.data_as(VP), g.n) == 0
    orc = H.CpuSystem("orc", P)
    _to_oracle(orc, g)
    orc.lib.orc_set_force(f.ctypes.data_as(VP))
    orc.correct(False)
    g.correct(False)
    pg, po = g.pairs(), orc.pairs()
    assert len(pg) > 100000
    np.testing.assert_array_equal(pg, po)
    np.testing.assert_array_equal(g.get("number"), orc.get("number"))
    np.testing.assert_array_equal(g.get("acc0"), orc.get("acc0"))
    assert rel_err(g.get("acc"), orc.get("acc")).max() < 1e-12
    # cluster formation
    g.cluster()
    orc.cluster()
    idc, num = g.get("id_cluster"), g.get("number")
    np.testing.assert_array_equal(idc, orc.get("id_cluster"))
    off, mem = g.cluster_lists()
    dev = {frozenset(mem[off[k]:off[k + 1]].tolist()) for k in range(len(off) - 1)}
    assert dev == _clusters_from(idc, num)
    assert len(dev) > 50000 and np.diff(off).max() >= 64
    # the hard part from identical states
    _to_oracle(orc, g)
    iso = g.get("number") == 0
    c_o, e_o = orc.hard(1)
    c_g, e_g = g.hard(1)
    np.testing.assert_array_equal(c_g, c_o)
    np.testing.assert_allclose(e_g, e_o, rtol=1e-9, atol=1e-30)
    for k in ("pos", "vel"):
        assert rel_err(g.get(k), orc.get(k)).max() < 1e-13, k
    np.testing.assert_array_equal(g.get("dead"), orc.get("dead"))
    np.testing.assert_array_equal(g.get("time"), orc.get("time"))
    dt_g, dt_o = g.get("dt"), orc.get("dt")
    diff = dt_g != dt_o
    assert not (diff & ~iso).any(), "a cluster member took a different block step"
    assert diff.mean() < 1e-3


def test_soft_neighbour_fields_at_1m_bodies(gpu):
    from gplum_gb300.radii import cutoff_radii
    from gplum_gb300.soft import epi_records, epj_records
    from gplum_gb300.tree import build_lists

    P = P3TParams(n_group_limit=256)
    d = disk_1m_soft(N, seed=2)
    r_out, r_search, _ = cutoff_radii(d["pos"], d["vel"], d["mass"], P)
    epj = epj_records(d["pos"], d["vel"], d["mass"], r_out, r_search, ids=d["id"])
    L = build_lists(d["pos"], d["mass"], r_search, P.theta, P.n_leaf_limit, P.n_group_limit)
    got = soft.soft_force_host(P, epj, L)
    H.CpuSystem("orc", P)
    lib = H.load("orc")
    epi = epi_records(epj)
    args = [L["n_group"]] + [L[k].ctypes.data_as(VP) for k in ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx")]
    f32 = cleared_forces(N)
    lib.orc_soft_lists(0, 0, *args, epi.ctypes.data_as(VP), epj.ctypes.data_as(VP), L["spj"].ctypes.data_as(VP),
                       f32.ctypes.data_as(VP), None, None, os.cpu_count())
    for k in ("number", "rank", "id_max", "id_min"):
        np.testing.assert_array_equal(got[k], f32[k], err_msg=k)
    acc4 = np.zeros(4 * N)
    ngb4 = np.zeros(4 * N, np.int32)
    lib.orc_soft_lists(1, 0, *args, epi.ctypes.data_as(VP), epj.ctypes.data_as(VP), L["spj"].ctypes.data_as(VP),
                       f32.ctypes.data_as(VP), acc4.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                       ngb4.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), os.cpu_count())
    a64 = acc4.reshape(N, 4)[:, :3]
    e_mixed = rel_err(got["acc"], a64)
    e_f32 = rel_err(f32["acc"], a64)
    assert np.median(e_mixed) <= 1e-6 and np.median(e_mixed) < np.median(e_f32)
    assert np.quantile(e_mixed, 0.99) < np.quantile(e_f32, 0.99)
