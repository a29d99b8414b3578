"""Shared set-up for the tests: seeded disks brought to a force-ready state by
the CPU oracle (start-up of src/main_p3t.cpp:289-364 of GPLUM), and their
FDPS records and interaction lists."""
import numpy as np

from gplum_gb300.disk import P3TParams, make_disk
from gplum_gb300.layout import EPI_DTYPE, EPJ_DTYPE
from gplum_gb300.tree import build_lists
from oracle import harness as H


def prepared_state(n=3000, seed=1, ecc_hill=2.0, inc_hill=1.0, a_in=0.95, a_out=1.05, m=1e-9, params=None,
                   with_acc_d=False):
    """Disk + radii (+ one start-up force pass for acc_d) via the oracle."""
    P = params or P3TParams()
    d = make_disk(n, m, a_in, a_out, ecc_hill=ecc_hill, inc_hill=inc_hill, seed=seed)
    s = H.CpuSystem("orc", P)
    s.load(d)
    s.f("set_r_planet")()
    s.prepare()
    if with_acc_d:
        lf = H.tree_lists_fn(P)
        s.soft_force(lf(s))
        s.correct(True)
    return P, d, s


def records(s):
    n = s.n
    epj = np.zeros(n, EPJ_DTYPE)
    epj["id_local"] = np.arange(n)
    epj["pos"] = s.get("pos")
    epj["r_out"] = s.get("r_out")
    epj["r_search"] = s.get("r_search")
    epj["id"] = s.get("id")
    epj["mass"] = s.get("mass")
    epj["vel"] = s.get("vel")
    epj["acc_d"] = s.get("acc_d")
    epi = np.zeros(n, EPI_DTYPE)
    for k in EPI_DTYPE.names:
        epi[k] = epj[k]
    return epi, epj


def lists_for(s, P, n_group_limit=None):
    return build_lists(s.get("pos"), s.get("mass"), s.get("r_search"), P.theta, P.n_leaf_limit,
                       n_group_limit or P.n_group_limit)


def rel_err(a, b):
    """Per-particle |a - b| / |b| for (n, 3) vectors."""
    num = np.sqrt(((np.asarray(a, float) - np.asarray(b, float)) ** 2).sum(-1))
    den = np.sqrt((np.asarray(b, float) ** 2).sum(-1))
    return num / np.maximum(den, 1e-300)
