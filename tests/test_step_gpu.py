"""The device-resident P3T step against the CPU oracle.

Bit-exact: neighbour counts, neighbour pairs, cluster labels and
memberships, collision pairs.  Tolerances (relative): accelerations that
include the FP32 soft part 1e-5 per body (1e-6 median); FP64-only
quantities from identical inputs 1e-12 (they differ from the host only
through log/sin/cos/atan2/pow/exp of the CUDA math library).
"""
import numpy as np
import pytest

from gplum_gb300.disk import P3TParams, make_disk
from gplum_gb300.p3t import GpuSystem
from oracle import harness as H
from tests.common import rel_err

pytestmark = pytest.mark.gpu

COPY = ("pos", "vel", "acc_d", "jerk_d", "acc_s", "jerk_s", "phi_s", "phi_d", "dt", "acc0", "time", "mass",
        "r_planet", "r_out", "r_out_inv", "r_search", "v_disp")


def both(disk, P):
    orc = H.CpuSystem("orc", P)
    gpu = GpuSystem(P)
    lf = H.tree_lists_fn(P)
    return orc, gpu, lf


def sync_state(src, dst, names=COPY):
    for k in names:
        dst.set(k, src.get(k))


def pair_set(s):
    return set(map(tuple, s.pairs().tolist()))


@pytest.mark.parametrize("seed,ecc", [(21, 4.0), (22, 8.0)])
def test_correction_neighbours_and_clusters(gpu, seed, ecc):
    P = P3TParams()
    d = make_disk(3000, 1e-9, 0.95, 1.05, ecc_hill=ecc, inc_hill=ecc / 2, seed=seed)
    orc, g, lf = both(d, P)
    for s in (orc, g):
        s.load(d)
        s.f("set_r_planet")()
        s.prepare()
    sync_state(orc, g, ("r_out", "r_out_inv", "r_search", "v_disp", "r_planet"))
    for initial in (True, True, False):
        L = lf(orc)
        orc.soft_force(L)
        g.soft_force(L)
        orc.correct(initial)
        g.correct(initial)
        np.testing.assert_array_equal(g.get("number"), orc.get("number"))
        assert pair_set(g) == pair_set(orc)
        e = rel_err(g.get("acc"), orc.get("acc"))
        assert np.median(e) < 1e-6 and e.max() < 1e-4, (np.median(e), e.max())
        if initial:
            for k in ("acc_d", "jerk_d"):
                num = np.abs(g.get(k) - orc.get(k)).max()
                assert num <= 1e-12 * max(np.abs(orc.get(k)).max(), 1e-300), k
            np.testing.assert_array_equal(g.get("dt"), orc.get("dt"))
        np.testing.assert_allclose(g.get("acc0"), orc.get("acc0"), rtol=1e-13)
        sync_state(orc, g, ("acc_d", "jerk_d", "phi_d", "dt", "acc0"))
    orc.cluster()
    g.cluster()
    np.testing.assert_array_equal(g.get("id_cluster"), orc.get("id_cluster"))
    # cluster lists: members of every cluster, ascending, clusters by smallest member
    off, mem = g.cluster_lists()
    num = orc.get("number")
    cid = orc.get("id_cluster")
    want = {}
    for i in np.nonzero(num)[0]:
        want.setdefault(cid[i], []).append(int(i))
    got = [list(mem[off[k]:off[k + 1]]) for k in range(len(off) - 1)]
    assert sorted(got) == sorted(want.values())
    assert all(c == sorted(c) for c in got)
    assert [c[0] for c in got] == sorted(c[0] for c in got)
    # the counts GPLUM logs at snapshot steps, from the device lists
    from gplum_gb300.run import cluster_counts, cluster_stats

    ids, sizes = np.unique(cid[num > 0], return_counts=True)
    assert cluster_stats(g) == cluster_counts(g.n, sizes, ids)


def test_hard_step_from_identical_states(gpu):
    P = P3TParams()
    d = make_disk(3000, 1e-9, 0.97, 1.03, ecc_hill=6.0, inc_hill=3.0, seed=23, f=60.0)
    orc, g, lf = both(d, P)
    H.p3t_init(orc, d, lf)
    H.p3t_init(g, d, lf)
    ncol = 0
    for istep in (1, 2, 3):
        orc.kick()
        g.kick()
        orc.cluster()
        g.cluster()
        np.testing.assert_array_equal(g.get("id_cluster"), orc.get("id_cluster"))
        sync_state(orc, g)
        g.set("id", orc.get("id"))
        iso = orc.get("number") == 0  # isolated bodies: Kepler drift
        c1, e1 = orc.hard(istep)
        c2, e2 = g.hard(istep)
        np.testing.assert_array_equal(c2, c1)
        ncol += len(c1)
        np.testing.assert_allclose(e2, e1, rtol=1e-9, atol=1e-30)
        for k in ("pos", "vel"):
            assert rel_err(g.get(k), orc.get(k)).max() < 1e-13, k
        for k in ("acc_d", "jerk_d", "acc_s", "jerk_s"):
            a, b = g.get(k), orc.get(k)
            assert np.abs(a - b).max() <= 1e-9 * np.abs(b).max(), k
        np.testing.assert_array_equal(g.get("dead"), orc.get("dead"))
        np.testing.assert_array_equal(g.get("n_cluster"), orc.get("n_cluster"))
        # block steps equal on every cluster member; an isolated body's step
        # (calcDeltatInitial after the Kepler drift, src/hermite.h:787-815) can
        # differ where CUDA's sin/cos/atan2 and glibc's round a drifted
        # position differently in the last bit
        dtg, dto = g.get("dt"), orc.get("dt")
        assert not ((dtg != dto) & ~iso).any()
        assert (dtg == dto).mean() > 0.999
        np.testing.assert_array_equal(g.get("time"), orc.get("time"))
        # finish the step identically on both (oracle state copied over);
        # local ids are refreshed after the merge removed the twins
        if len(c1):
            orc.merge(len(c1))
            g.merge(len(c2))
            assert g.n == orc.n
            np.testing.assert_array_equal(g.get("id"), orc.get("id"))
        for s in (orc, g):
            s.f("set_id_local")()
        L = lf(orc)
        sync_state(orc, g)
        g.set("id", orc.get("id"))
        for s in (orc, g):
            s.soft_force(L)
            s.correct(False)
            s.kick()
        sync_state(orc, g)
    assert ncol > 0


def test_full_steps_track_the_oracle(gpu):
    P = P3TParams()
    d = make_disk(3000, 1e-9, 0.95, 1.05, ecc_hill=2.0, inc_hill=1.0, seed=1)
    orc, g, lf = both(d, P)
    e0o = H.p3t_init(orc, d, lf)
    e0g = H.p3t_init(g, d, lf)
    assert abs(e0g[0] - e0o[0]) <= 1e-9 * abs(e0o[0])
    for istep in range(1, 11):
        a = H.p3t_step(orc, istep, lf)
        b = H.p3t_step(g, istep, lf)
        np.testing.assert_array_equal(b["cols"], a["cols"])
        assert a["n_clusters"] == b["n_clusters"]
        assert rel_err(g.get("pos"), orc.get("pos")).max() < 1e-10
        dEo = (a["energy"][0] - e0o[0]) / e0o[0]
        dEg = (b["energy"][0] - e0g[0]) / e0g[0]
        assert abs(dEg - dEo) < 1e-9, (dEg, dEo)


def test_isolated_bodies_take_the_sun_hermite(gpu):
    """With a softened sun (eps2_sun > 0) isolated bodies are integrated by the
    sun-only block-step Hermite (src/hermite.h:734-785) instead of the Kepler
    drift (src/hard.h:803-811); cluster members feel the softened sun too."""
    P = P3TParams(eps2_sun=1e-6)
    d = make_disk(3000, 1e-9, 0.95, 1.05, ecc_hill=2.0, inc_hill=1.0, seed=24)
    orc, g, lf = both(d, P)
    H.p3t_init(orc, d, lf)
    H.p3t_init(g, d, lf)
    for istep in (1, 2):
        orc.kick()
        g.kick()
        orc.cluster()
        g.cluster()
        sync_state(orc, g)
        g.set("id", orc.get("id"))
        c1, _ = orc.hard(istep)
        c2, _ = g.hard(istep)
        np.testing.assert_array_equal(c2, c1)
        iso = orc.get("n_cluster") == 1
        assert iso.sum() > 1000
        for k in ("pos", "vel"):
            assert rel_err(g.get(k), orc.get(k)).max() < 1e-13, k
        np.testing.assert_array_equal(g.get("dt")[iso], orc.get("dt")[iso])
        np.testing.assert_array_equal(g.get("time"), orc.get("time"))
        for s in (orc, g):
            s.f("set_id_local")()
        L = lf(orc)
        sync_state(orc, g)
        for s in (orc, g):
            s.soft_force(L)
            s.correct(False)
            s.kick()
        sync_state(orc, g)


def test_out_of_boundary_removal(gpu):
    """removeParticlesOutOfBoundary on the device: the same bodies leave and
    take the same energy (to 1e-12) as in the restatement."""
    P = P3TParams()
    d = make_disk(3000, 1e-9, 0.95, 1.05, ecc_hill=3.0, inc_hill=1.5, seed=42)
    orc, g, lf = both(d, P)
    H.p3t_init(orc, d, lf)
    H.p3t_init(g, d, lf)
    sync_state(orc, g)
    r = np.sqrt((orc.get("pos") ** 2).sum(1))
    r_min, r_max = np.quantile(r, 0.03), np.quantile(r, 0.96)
    n1, e1 = orc.remove(r_max, r_min)
    n2, e2 = g.remove(r_max, r_min)
    assert n1 == n2 > 100
    assert abs(e2 - e1) <= 1e-12 * abs(e1)
    np.testing.assert_array_equal(g.get("id"), orc.get("id"))
    np.testing.assert_array_equal(g.get("pos"), orc.get("pos"))
    assert g.n == orc.n == 3000 - n1


def test_no_clusters(gpu):
    """A sparse system in which no body has a neighbour: no clusters, an empty
    hard queue, every body on the Kepler drift; three steps against the
    oracle."""
    P = P3TParams()
    d = make_disk(200, 1e-12, 0.5, 1.5, ecc_hill=2.0, inc_hill=1.0, seed=27)
    orc, g, lf = both(d, P)
    H.p3t_init(orc, d, lf)
    H.p3t_init(g, d, lf)
    assert orc.get("number").max() == 0
    for istep in (1, 2, 3):
        a = H.p3t_step(orc, istep, lf)
        b = H.p3t_step(g, istep, lf)
        assert a["n_clusters"] == b["n_clusters"] == 0
        assert len(a["cols"]) == len(b["cols"]) == 0
        assert rel_err(g.get("pos"), orc.get("pos")).max() < 1e-12
        np.testing.assert_array_equal(g.get("number"), orc.get("number"))
    off, _ = g.cluster_lists()
    assert len(off) == 1
