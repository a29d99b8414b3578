"""Interaction lists of the host tree (the FDPS LONG_SYMMETRY contract)."""
import numpy as np

from tests.common import lists_for, prepared_state


def test_lists_cover_search_radius_and_partition():
    P, d, s = prepared_state(n=4000, seed=3, ecc_hill=4.0, inc_hill=2.0)
    L = lists_for(s, P)
    n = s.n
    pos, rs, mass = s.get("pos"), s.get("r_search"), s.get("mass")
    # every particle in exactly one group, groups within the limit
    assert np.array_equal(np.sort(L["i_idx"]), np.arange(n))
    sizes = np.diff(L["i_off"])
    assert sizes.min() >= 1 and sizes.max() <= P.n_group_limit
    # total mass seen by each group: its EPJ + SPJ masses = system mass
    tot = mass.sum()
    for g in range(0, L["n_group"], 7):
        jm = mass[L["j_idx"][L["j_off"][g]:L["j_off"][g + 1]]].sum()
        sm = L["spj"]["mass"][L["s_idx"][L["s_off"][g]:L["s_off"][g + 1]]].sum()
        assert abs(jm + sm - tot) <= 1e-12 * tot
    # the symmetric search rule: j within max(1.1 rs_i, 1.1 rs_j) of i is an EPJ of i's group
    for g in range(0, L["n_group"], 5):
        ii = L["i_idx"][L["i_off"][g]:L["i_off"][g + 1]]
        jj = set(L["j_idx"][L["j_off"][g]:L["j_off"][g + 1]].tolist())
        for i in ii:
            dr = np.sqrt(((pos - pos[i]) ** 2).sum(1))
            near = np.nonzero(dr < np.maximum(1.1 * rs[i], 1.1 * rs))[0]
            assert set(near.tolist()) <= jj


def test_single_particle_and_tiny_groups():
    P, d, s = prepared_state(n=5, seed=4)
    L = lists_for(s, P, n_group_limit=1)
    assert L["n_group"] == 5
    assert np.array_equal(np.sort(L["i_idx"]), np.arange(5))


def test_thin_disk_with_off_centre_bodies_keeps_groups_compact():
    """Embryos on inclined orbits move the bodies' bounding box off the disk's
    mid-plane.  The root cube is anchored at the bodies' lower corner, so the
    thin axis is not cut through the disk at coarse levels: no group spreads
    over a wide patch of the disk (a cut near the mid-plane would leave sparse
    groups of the few bodies above it, each as wide as a coarse cell, with
    EPJ lists of tens of thousands)."""
    from gplum_gb300.disk import P3TParams, disk_1m_embryos
    from gplum_gb300.radii import cutoff_radii
    from gplum_gb300.tree import build_lists

    P = P3TParams(n_group_limit=256)
    d = disk_1m_embryos()  # 1,048,576 planetesimals + 4 embryos (a few seconds on the host)
    ro, rs, _ = cutoff_radii(d["pos"], d["vel"], d["mass"], P)
    L = build_lists(d["pos"], d["mass"], rs, P.theta, P.n_leaf_limit, P.n_group_limit)
    pos = d["pos"]
    assert 0.5 * (pos[:, 2].max() + pos[:, 2].min()) > 1e-3  # the box is off the mid-plane
    box = np.array([np.ptp(pos[L["i_idx"][L["i_off"][g]:L["i_off"][g + 1]], :2], axis=0).max()
                    for g in range(L["n_group"])])
    assert box.max() < 0.15  # groups of <= 256 of a million bodies; a coarse-level cut gave 0.37 AU
    nj = np.diff(L["j_off"])
    assert nj.max() < 5 * np.median(nj)  # a coarse-level cut gave 38,049 against a median of 417
