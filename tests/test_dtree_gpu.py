"""The device octree and interaction lists against the host builder.

The device build (gplum_gb300/csrc/dtree.cu) follows the host builder's
contract and traversal order, so for the same bodies:
  - groups and their members are identical (Morton order, same cells);
  - every group's EPJ list is identical, entry for entry;
  - every group's SPJ list names the same cells in the same order: the
    records agree exactly in mass for leaves and to 1e-12 relative otherwise
    (inner moments combine children by the parallel-axis rule instead of
    summing bodies in key order);
  - the soft force from the device lists equals the one from the host lists
    to 1e-6 relative, with identical neighbour counts.
"""
import ctypes

import numpy as np
import pytest

from gplum_gb300.disk import P3TParams, disk_3000, make_disk
from gplum_gb300.layout import FORCE_DTYPE
from gplum_gb300.p3t import GpuSystem
from gplum_gb300.tree import build_lists
from tests.common import rel_err

pytestmark = pytest.mark.gpu


def prepared(d, ngl):
    P = P3TParams(n_group_limit=ngl)
    g = GpuSystem(P)
    g.load(d)
    g.set_r_planet()
    g.prepare()
    return g, P


def host_lists(g, P):
    return build_lists(g.get("pos"), g.get("mass"), g.get("r_search"), P.theta, P.n_leaf_limit, P.n_group_limit)


CASES = [
    ("3000", lambda: disk_3000(), 64),
    ("65k soft disk", lambda: make_disk(65536, 1e-10 * 16, 0.5, 1.5, seed=12), 256),
    ("131k hard disk", lambda: make_disk(131072, 7e-11 * 8 ** 1.5, 0.95, 1.05, ecc_hill=6.0, inc_hill=3.0,
                                         seed=13), 256),
]


@pytest.mark.parametrize("walk", [1, 0], ids=["breadth-first", "tasks"])
@pytest.mark.parametrize("name,mk,ngl", CASES)
def test_device_lists_equal_host_lists(gpu, name, mk, ngl, walk):
    g, P = prepared(mk(), ngl)
    H = host_lists(g, P)
    assert g.lib.p3t_set_walk(walk) == 0
    try:
        D = g.tree_lists(build=True)
        assert g.lib.p3t_walk_last() == walk
    finally:
        g.lib.p3t_set_walk(1)
    assert D["n_group"] == H["n_group"]
    for k in ("i_off", "i_idx", "j_off", "j_idx", "s_off"):
        np.testing.assert_array_equal(D[k], H[k], err_msg=k)
    hs, ds = H["spj"][H["s_idx"]], D["spj"][D["s_idx"]]
    np.testing.assert_allclose(ds["mass"], hs["mass"], rtol=1e-12, atol=0)
    # centres of mass sum in a different association order: compare each
    # component at 1e-12 of the position scale (a component near 0 keeps the
    # absolute rounding of the O(1) terms it cancels)
    np.testing.assert_allclose(ds["pos"], hs["pos"], rtol=1e-12, atol=1e-12 * np.abs(hs["pos"]).max())
    q = np.stack([hs[k] for k in ("xx", "yy", "zz", "xy", "xz", "yz")], 1)
    qd = np.stack([ds[k] for k in ("xx", "yy", "zz", "xy", "xz", "yz")], 1)
    scale = np.abs(q[:, :3]).max(1, keepdims=True) + 1e-300
    assert (np.abs(qd - q) / scale).max() < 1e-9


def soft_out(g):
    f = np.zeros(g.n, FORCE_DTYPE)
    g._chk(g.lib.p3t_download_forces(f.ctypes.data_as(ctypes.c_void_p), g.n), "p3t_download_forces")
    return f


@pytest.mark.parametrize("name,mk,ngl", CASES[:2])
def test_soft_force_from_device_lists(gpu, name, mk, ngl):
    g, P = prepared(mk(), ngl)
    g.soft_force(host_lists(g, P))
    fh = soft_out(g)
    g.tree_soft()
    fd = soft_out(g)
    for k in ("number", "rank", "id_max", "id_min"):
        np.testing.assert_array_equal(fd[k], fh[k], err_msg=k)
    assert rel_err(fd["acc"].astype(np.float64), fh["acc"].astype(np.float64)).max() < 1e-6
    assert (np.abs(fd["phi"] - fh["phi"]) / np.abs(fh["phi"])).max() < 1e-6


# both walk forms and both moment forms (form bit 1: one launch per level) on
# the 1M-body hard-part disk: the same lists entry for entry, the same cells
def test_walk_forms_agree_at_1m(gpu):
    from gplum_gb300.disk import disk_1m_hard

    g, P = prepared(disk_1m_hard(1048576), 256)
    out = []
    try:
        for form in (1, 0, 3):
            assert g.lib.p3t_set_walk(form) == 0
            out.append(g.tree_lists(build=True))
            assert g.lib.p3t_walk_last() == form & 1
    finally:
        g.lib.p3t_set_walk(1)
    a = out[0]
    for b in out[1:]:
        for k in ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx"):
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
        assert a["spj"].tobytes() == b["spj"].tobytes()


# the breadth-first walk's fallbacks: a frontier above the CTA's limit, or a
# frontier store too small for the build, hands the build to the task walk,
# with the same lists; the store grows by itself for the next build
@pytest.mark.parametrize("cap,store", [(8, 0), (4096, 1000)])
def test_walk_fallback_same_lists(gpu, cap, store):
    name, mk, ngl = CASES[1]
    g, P = prepared(mk(), ngl)
    H = host_lists(g, P)
    try:
        assert g.lib.p3t_set_walk_limits(cap, store) == 0
        D = g.tree_lists(build=True)
        assert g.lib.p3t_walk_last() == 0
        for k in ("i_off", "i_idx", "j_off", "j_idx", "s_off"):
            np.testing.assert_array_equal(D[k], H[k], err_msg=k)
        if store:
            D2 = g.tree_lists(build=True)  # the store grew: breadth first again
            assert g.lib.p3t_walk_last() == 1
            for k in ("j_idx", "s_idx"):
                np.testing.assert_array_equal(D2[k], D[k], err_msg=k)
    finally:
        g.lib.p3t_set_walk_limits(4096, 1 << 24)
