"""The two execution forms of the hard launch give bit-identical results.

Bundles (many clusters per CTA, FP32 pair prefilter with proven margins,
FP64 pair terms folded in partner order) against the thread/warp/CTA tiers
(one cluster per team, FP64 pair loop): the same device state, restored from
a snapshot, integrated once by each, must agree bit for bit in every body
field, the collision list, the dissipated energy and the per-cluster cost log
(block steps and pair sweeps).  The tier form itself is checked against the
CPU oracle in test_step_gpu.py.
"""
import ctypes

import numpy as np
import pytest

from gplum_gb300.disk import P3TParams, make_disk
from gplum_gb300.p3t import GpuSystem
from gplum_gb300.tree import build_lists

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "acc_d", "jerk_d", "acc_s", "jerk_s", "phi_s", "phi_d", "dt", "time", "mass", "r_planet",
          "id", "dead", "merged", "n_cluster")


def prepared(n, f, seed, mfac=1.0):
    """The 0.95-1.05 AU disk with rms e = 6 h, rms i = 3 h and the body mass of
    the hard-part workload at this n (7e-11 at 1,048,576 bodies, scaled n^-1.5,
    times mfac); f inflates the collision radii to force collisions."""
    P = P3TParams(n_group_limit=256)
    m = 7e-11 * (1048576.0 / n) ** 1.5 * mfac
    d = make_disk(n, m, 0.95, 1.05, ecc_hill=6.0, inc_hill=3.0, seed=seed, f=f)
    g = GpuSystem(P)
    g.load(d)
    g.set_r_planet()
    g.prepare()
    for _ in range(2):
        L = build_lists(g.get("pos"), g.get("mass"), g.get("r_search"), P.theta, P.n_leaf_limit, P.n_group_limit)
        g.soft_force(L)
        g.correct(True)
    g.kick()
    g.cluster()
    return g


def run(g, mode, nc):
    g.lib.p3t_set_hard_mode(mode)
    assert g.lib.p3t_state_snapshot(1) == 0
    cols, ed = g.hard(1)
    cost = np.zeros(2 * nc, np.int64)
    assert g.lib.p3t_hard_costs(cost.ctypes.data_as(ctypes.c_void_p), nc) == 0
    return cols, ed, {k: g.get(k) for k in FIELDS}, cost


# the last two: heavier bodies near percolation give clusters of 257-512 bodies
# (the wide lone bundles) and, with mfac 2, of more than 512 (the
# one-cluster-per-CTA form inside the wide launch)
@pytest.mark.parametrize("n,f,seed,mfac", [(65536, 1.0, 5, 1.0), (65536, 40.0, 6, 1.0), (8192, 200.0, 7, 1.0),
                                           (16384, 30.0, 8, 1.5), (16384, 1.0, 8, 2.0)])
def test_bundles_match_tiers_bitwise(gpu, n, f, seed, mfac):
    g = prepared(n, f, seed, mfac)
    off, _ = g.cluster_lists()
    nc = len(off) - 1
    assert nc > 100
    if mfac > 1.0:
        assert np.diff(off).max() > (512 if mfac >= 2.0 else 256)
    assert g.lib.p3t_state_snapshot(0) == 0
    try:
        t = run(g, 1, nc)
        forms = []
        # bundle shapes and placements of the clusters above the slots
        for cap, occ, wide in ((256, 2, 1), (256, 2, 0), (128, 3, 1)):
            assert g.lib.p3t_set_hard_bundle(cap, occ) == 0
            assert g.lib.p3t_set_hard_wide(wide) == 0
            forms.append(run(g, 0, nc))
    finally:
        g.lib.p3t_set_hard_mode(0)
        g.lib.p3t_set_hard_wide(0)
        g.lib.p3t_set_hard_bundle(256, 2)
    for b in forms:
        np.testing.assert_array_equal(b[0], t[0])
        assert b[1].tobytes() == t[1].tobytes()
        for k in FIELDS:
            assert b[2][k].tobytes() == t[2][k].tobytes(), k
        np.testing.assert_array_equal(b[3], t[3])
    b = forms[0]
    if f > 1.0:
        assert len(b[0]) > 0


# the lone form (one cluster per CTA, the whole cluster in shared memory) for
# the clusters the learned model predicts to run longest, in CTAs of its own
# (ctas > 0) and inside the bundle kernel's CTAs (ctas = 0): with a threshold
# of 0.5 every cluster of at most 64 members goes there, with 3.0 the head of
# the queue; collisions (f > 1) hand a cluster to the one-cluster-per-team loop
# mid-integration
@pytest.mark.parametrize("n,f,seed", [(65536, 1.0, 5), (65536, 40.0, 6), (8192, 200.0, 7)])
def test_lone_form_matches_tiers_bitwise(gpu, n, f, seed):
    from gplum_gb300 import scheduler

    g = prepared(n, f, seed)
    off, _ = g.cluster_lists()
    nc = len(off) - 1
    assert g.lib.p3t_state_snapshot(0) == 0
    scheduler.load(lib=g.lib)
    assert g.lib.p3t_set_schedule(1) == 0
    try:
        t = run(g, 1, nc)
        forms = []
        for thr, ctas in ((0.5, 152), (3.0, 16), (0.5, 0), (3.0, 0)):
            assert g.lib.p3t_set_hard_lone(thr, ctas) == 0
            forms.append(run(g, 0, nc))
    finally:
        g.lib.p3t_set_hard_lone(0.0, 0)
        g.lib.p3t_set_schedule(0)
        g.lib.p3t_set_hard_mode(0)
    for b in forms:
        np.testing.assert_array_equal(b[0], t[0])
        assert b[1].tobytes() == t[1].tobytes()
        for k in FIELDS:
            assert b[2][k].tobytes() == t[2][k].tobytes(), k
        np.testing.assert_array_equal(b[3], t[3])
    if f > 1.0:
        assert len(forms[0][0]) > 0
