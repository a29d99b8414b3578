"""Failure detection on the GPU without a GPU fault.  Every device loop of
the library writes a status bit instead of trapping; each case below makes
one bit fire on purpose with an input the kernels handle safely, checks the
status the host reads back, and checks that the library keeps working
afterwards (GPLUM stops with PS::Abort / assert on the same conditions,
src/main_p3t.cpp:160-203,528-529).

* 2 -- a list entry out of range: the soft kernel clamps it before the load;
* 1 -- more neighbour candidates than the table holds: the correction widens
  the table and runs the soft pass again, with results identical to a run
  that never overflowed;
* 4 -- a cluster reaches the block-step cap (lowered by
  p3t_set_hard_step_cap): it stops there and the launch ends;
* 16 -- a fragmenting collision in a cluster above the bundle's 256 member
  slots (the one-cluster-per-CTA form does not place fragments): the
  collision merges without fragments.
"""
import numpy as np
import pytest

from gplum_gb300 import _lib, soft
from gplum_gb300.disk import P3TParams, make_disk
from gplum_gb300.p3t import GpuSystem
from tests.common import lists_for, prepared_state, records, rel_err

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "acc", "acc_d", "jerk_d", "dt", "id_cluster", "number")


def test_out_of_range_list_entry_reports_bad_index(gpu):
    P, d, s = prepared_state(n=2000, seed=31, ecc_hill=4.0, inc_hill=2.0)
    epi, epj = records(s)
    L = lists_for(s, P)
    sf = soft.SoftForce(P)
    lib = sf.lib
    assert lib.p3t_status() == 0
    sf.upload_particles(epj)
    bad = dict(L)
    bad["j_idx"] = L["j_idx"].copy()
    bad["j_idx"][0] = len(epj) + 5
    bad["s_idx"] = L["s_idx"].copy()
    bad["s_idx"][-1] = len(L["spj"])
    sf.upload_lists(bad)
    sf.run()
    sf.synchronize()
    assert lib.p3t_status() == 2
    assert lib.p3t_status() == 0  # read and cleared
    sf.upload_lists(L)
    sf.run()
    got = sf.download()
    want = soft.soft_force_host(P, epj, L)
    for k in ("number", "rank", "id_max", "id_min"):
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    assert rel_err(got["acc"], want["acc"]).max() <= 1e-6


def _run(P, d, cand_cap, steps=2):
    g = GpuSystem(P, cand_cap=cand_cap)
    g.load(d)
    g.set_r_planet()
    g.startup()
    for istep in range(1, steps + 1):
        g.tree_step(istep)
    return {k: g.get(k) for k in FIELDS}


def test_candidate_overflow_widens_the_table_and_repeats(gpu):
    P = P3TParams()
    d = make_disk(3000, 1e-9, 0.97, 1.03, ecc_hill=4.0, inc_hill=2.0, seed=32)
    want = _run(P, d, 64)
    got = _run(P, d, 1)  # every body with two or more screen hits overflows the first pass
    for k in FIELDS:
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    # back to the default table for the tests that follow
    soft.configure(P, 0, 0, 64)


def test_block_step_cap_stops_the_cluster_and_reports(gpu):
    P = P3TParams()
    d = make_disk(3000, 1e-9, 0.97, 1.03, ecc_hill=4.0, inc_hill=2.0, seed=33)
    g = GpuSystem(P)
    g.load(d)
    g.set_r_planet()
    g.startup()
    lib = g.lib
    try:
        assert lib.p3t_set_hard_step_cap(2) == 0
        g.kick()
        g.cluster()
        with pytest.raises(RuntimeError, match="kernel status bits 4"):
            g.hard(1)
    finally:
        assert lib.p3t_set_hard_step_cap(1 << 20) == 0
    assert lib.p3t_status() == 0
    # the library runs the same disk normally afterwards
    g.load(d)
    g.set_r_planet()
    g.startup()
    r = g.tree_step(1)
    assert np.isfinite(g.get("pos")).all() and r["n_body"] == g.n


def _ring_with_a_collision(n=300):
    """n bodies of 1e-9 on one circular orbit, 1e-3 AU apart (each within
    the neighbour radius of the next: one cluster of n), and one more body
    3e-6 AU from the first.  The pair's radii are enlarged 500 times (GPLUM's
    increase factor f) to 2e-3 AU: their mutual pull carries them ~4e-4 AU
    past each other within the first block step, and collisions are tested
    only at block-step times, so the radii must cover that motion."""
    ang = np.arange(n) * 1e-3
    a = 1.0
    pos = np.stack([a * np.cos(ang), a * np.sin(ang), np.zeros(n)], 1)
    vel = np.stack([-np.sin(ang), np.cos(ang), np.zeros(n)], 1) / np.sqrt(a)
    pos = np.vstack([pos, pos[:1] + [0.0, 0.0, 3e-6]])
    vel = np.vstack([vel, vel[:1]])
    m = np.full(n + 1, 1e-9)
    f = np.ones(n + 1)
    f[0] = f[n] = 500.0
    return {"id": np.arange(n + 1, dtype=np.int64), "mass": m, "r_planet": np.zeros(n + 1), "f": f,
            "pos": pos, "vel": vel}


def test_fragmenting_collision_in_an_oversized_cluster_reports(gpu):
    P = P3TParams()
    d = _ring_with_a_collision()
    g = GpuSystem(P)
    lib = g.lib
    assert lib.p3t_set_hard_mode(0) == 0 and lib.p3t_set_hard_wide(0) == 0
    g.set_fragmentation(0.5)
    try:
        g.load(d)
        g.set_r_planet()
        g.startup()
        g.kick()
        g.cluster()
        off, _m = g.cluster_lists()
        assert np.diff(off).max() > 256
        with pytest.raises(RuntimeError, match="kernel status bits 16"):
            g.hard(1)
    finally:
        g.set_fragmentation(0.0)
    assert lib.p3t_status() == 0
    # the collision merged without fragments: no body joined the system
    recs = g.collisions()
    assert len(recs) >= 1 and g.n == len(d["mass"])
    assert {0, len(d["mass"]) - 1} & set(recs.ravel().tolist())
