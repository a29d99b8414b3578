"""The CPU oracle against fixtures produced by GPLUM's own code
(tests/golden/make_golden.py): bit-exact on every field."""
import ctypes
import os

import numpy as np
import pytest

from gplum_gb300.disk import P3TParams
from gplum_gb300.layout import EPI_DTYPE, EPJ_DTYPE, FORCE_DTYPE, SPJ_DTYPE, cleared_forces
from oracle import harness as H

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _params(vec):
    names = ["eps2", "eps2_sun", "m_sun", "dt_tree", "dt_min", "eta", "eta_0", "eta_sun", "eta_sun0", "alpha2",
             "gamma", "R_cut0", "R_cut1", "R_search0", "R_search1", "R_search2", "R_search3", "r_cut_min",
             "r_cut_max", "p_cut", "dens"]
    return P3TParams(**dict(zip(names, [float(x) for x in vec])))


def test_soft_functors_bit_exact():
    z = np.load(os.path.join(GOLD, "soft_functor.npz"))
    P = _params(z["params"])
    H.CpuSystem("orc", P)  # sets the oracle's parameters
    lib = H.load("orc")
    epj = z["epj"].view(EPJ_DTYPE)
    spj = z["spj"].view(SPJ_DTYPE)
    want = z["force"].view(FORCE_DTYPE)
    epi = np.zeros(len(epj), EPI_DTYPE)
    for k in EPI_DTYPE.names:
        epi[k] = epj[k]
    i_off, i_idx, j_off, j_idx, s_off, s_idx = (z[k] for k in ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx"))
    got = cleared_forces(len(epj))
    for g in range(len(i_off) - 1):
        ii = i_idx[i_off[g]:i_off[g + 1]]
        ei = np.ascontiguousarray(epi[ii])
        ej = np.ascontiguousarray(epj[j_idx[j_off[g]:j_off[g + 1]]])
        sj = np.ascontiguousarray(spj[s_idx[s_off[g]:s_off[g + 1]]])
        f = cleared_forces(len(ii))
        vp = ctypes.c_void_p
        lib.orc_epep_f32(ei.ctypes.data_as(vp), len(ei), ej.ctypes.data_as(vp), len(ej), f.ctypes.data_as(vp))
        lib.orc_epsp_f32(ei.ctypes.data_as(vp), len(ei), sj.ctypes.data_as(vp), len(sj), f.ctypes.data_as(vp), 0)
        got[ii] = f
    assert got.tobytes() == want.tobytes()


def test_scalars_bit_exact():
    z = np.load(os.path.join(GOLD, "scalars.npz"))
    s = H.CpuSystem("orc", _params(z["params"]))
    lib = s.lib
    consts = np.zeros(5)
    lib.orc_get_gamma_consts(consts.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    np.testing.assert_array_equal(consts, z["gamma_consts"])
    np.testing.assert_array_equal([lib.orc_cutoff_W(x, 1.0) for x in z["r"]], z["W"])
    np.testing.assert_array_equal([lib.orc_cutoff_K(x, 1.0) for x in z["r"]], z["K"])
    np.testing.assert_array_equal([lib.orc_cutoff_dKdt(x, 1.0, 0.3) for x in z["r"]], z["dKdt"])
    U = np.array([[lib.orc_solve_kepler(a, b) for a in z["l"]] for b in z["ecc"]])
    np.testing.assert_array_equal(U, z["u"])


def test_p3t_steps_bit_exact():
    """Start-up and four tree steps with collisions (perfect accretion)."""
    z = np.load(os.path.join(GOLD, "p3t_steps.npz"))
    P = _params(z["params"])
    s = H.CpuSystem("orc", P)
    disk = {k[5:]: z[k] for k in z.files if k.startswith("disk_")}
    lf = H.tree_lists_fn(P)
    e0 = H.p3t_init(s, disk, lf)
    np.testing.assert_array_equal(e0, z["e0"])

    def check(tag):
        for k in ("pos", "vel", "acc", "acc_d", "jerk_d", "phi", "phi_d", "dt", "acc0", "mass", "r_out",
                  "r_search", "id", "id_cluster", "number", "n_cluster"):
            np.testing.assert_array_equal(s.get(k), z[f"{tag}_{k}"], err_msg=f"{tag} {k}")
        assert set(map(tuple, s.pairs().tolist())) == set(map(tuple, z[f"{tag}_pairs"].tolist()))
        np.testing.assert_array_equal(s.energy(), z[f"{tag}_energy"])

    check("init")
    ncol = 0
    for st in range(1, 5):
        out = H.p3t_step(s, st, lf)
        np.testing.assert_array_equal(out["cols"], z[f"s{st}_cols"])
        np.testing.assert_array_equal(out["edisp"], z[f"s{st}_edisp"])
        ncol += len(out["cols"])
        check(f"s{st}")
    assert ncol == int(z["ncol"]) and ncol > 0
