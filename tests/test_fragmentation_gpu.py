"""KOMINAMI fragmentation on the device against the restatement (whose
fragment model is pinned to GPLUM's own build in test_fragment_pin.py).

From identical states, each tree step's hard part must give the same
collision list (temporary fragment ids included), the same number of new
bodies in the same order with the same new ids, and the same state to
1e-12 relative (positions and velocities go through the CUDA and host
libm's pow/sin/cos); the merge that follows must leave the same bodies.
"""
import ctypes

import numpy as np
import pytest

from gplum_gb300 import collisions
from gplum_gb300.disk import P3TParams, make_disk
from gplum_gb300.p3t import GpuSystem
from oracle import harness as H
from tests.common import rel_err

pytestmark = pytest.mark.gpu

COPY = ("pos", "vel", "acc_d", "jerk_d", "acc_s", "jerk_s", "phi_s", "phi_d", "dt", "acc0", "time", "mass",
        "r_planet", "r_out", "r_out_inv", "r_search", "v_disp")


def sync_state(src, dst):
    for k in COPY:
        dst.set(k, src.get(k))
    dst.set("id", src.get("id"))


def test_fragmenting_collisions_match_the_oracle(gpu):
    P = P3TParams()
    d = make_disk(3000, 1e-9, 0.97, 1.03, ecc_hill=6.0, inc_hill=3.0, seed=23, f=60.0)
    orc, g = H.CpuSystem("orc", P), GpuSystem(P)
    lf = H.tree_lists_fn(P)
    frag = dict(a_frag=0.5, n_frag=6, m_min=1e-10, seed=11)
    orc.set_fragmentation(**frag)
    g.set_fragmentation(**frag)
    try:
        H.p3t_init(orc, d, lf)
        H.p3t_init(g, d, lf)
        assert g.id_next() == orc.id_next() == 3000
        n_frag_total = 0
        for istep in (1, 2, 3):
            orc.kick()
            g.kick()
            orc.cluster()
            g.cluster()
            np.testing.assert_array_equal(g.get("id_cluster"), orc.get("id_cluster"))
            sync_state(orc, g)
            c1, e1 = orc.hard(istep)
            c2, e2 = g.hard(istep)
            np.testing.assert_array_equal(c2, c1)
            np.testing.assert_allclose(e2, e1, rtol=1e-9, atol=1e-30)
            # the collision-file records (final ids; masses, states before the
            # collision, centre-of-mass shifts)
            recs = collisions.records(g.lib)
            assert len(recs) == len(c1)
            for k, r in enumerate(recs):
                o = np.zeros(25)
                orc.lib.orc_col_record(k, o.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
                assert (r.id_imp, r.id_tar, r.n_frag, r.id_frag, r.flag) == tuple(int(x) for x in o[[1, 2, 3, 4, 20]])
                assert r.time == o[0]
                got = np.array([r.mass_imp, r.mass_tar, r.mass_frag, *r.pos_imp, *r.pos_tar, *r.vel_imp, *r.vel_tar])
                np.testing.assert_allclose(got, o[5:20], rtol=1e-12, atol=0)
                # the shifts are rounding-level differences of O(1) values
                assert abs(r.dpos_g_rel - o[21]) <= 1e-13 and abs(r.dvel_g_rel - o[22]) <= 1e-13
            assert g.n == orc.n
            n_frag_total += g.n - 3000 if istep == 1 else 0
            assert g.id_next() == orc.id_next()
            np.testing.assert_array_equal(g.get("id"), orc.get("id"))
            for k in ("pos", "vel"):
                assert rel_err(g.get(k), orc.get(k)).max() < 1e-12, k
            for k in ("mass", "r_planet"):
                np.testing.assert_allclose(g.get(k), orc.get(k), rtol=1e-13, atol=0)
            for k in ("dead", "merged", "n_cluster", "number"):
                np.testing.assert_array_equal(g.get(k), orc.get(k), err_msg=k)
            np.testing.assert_array_equal(g.get("time"), orc.get("time"))
            if len(c1):
                orc.merge(len(c1))
                g.merge(len(c2))
                assert g.n == orc.n
                np.testing.assert_array_equal(g.get("id"), orc.get("id"))
                np.testing.assert_allclose(g.get("mass"), orc.get("mass"), rtol=1e-13, atol=0)
            for s in (orc, g):
                s.f("set_id_local")()
            L = lf(orc)
            sync_state(orc, g)
            for s in (orc, g):
                s.prepare()
                s.soft_force(L)
                s.correct(True)
                s.kick()
            sync_state(orc, g)
        assert orc.id_next() > 3000, "no fragments were made"
    finally:
        orc.set_fragmentation(0.0)
        g.set_fragmentation(0.0)
