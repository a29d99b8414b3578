"""Generates the golden fixtures in this folder from GPLUM's own code.

Runs the reference build (oracle/_ref/libgplum_ref.so: GPLUM's hot-path
headers compiled unchanged against the single-rank PS shim) on seeded
synthetic inputs and stores inputs and outputs as .npz files.  Needs the
reference source tree, so it runs where that tree is mounted:

    python tests/golden/make_golden.py

The fixtures are small (a few hundred kB in total) and are what the CPU tests
pin the oracle against on machines without the reference tree.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gplum_gb300.disk import P3TParams, make_disk  # noqa: E402
from gplum_gb300.layout import EPI_DTYPE, EPJ_DTYPE, cleared_forces  # noqa: E402
from gplum_gb300.tree import build_lists  # noqa: E402
from oracle import harness as H  # noqa: E402


def soft_functor_fixture():
    """Per-group functor outputs (EP-EP then EP-SP into cleared records)."""
    P = P3TParams()
    d = make_disk(1200, 1e-9, 0.97, 1.03, ecc_hill=2.0, inc_hill=1.0, seed=11)
    ref = H.CpuSystem("ref", P)
    ref.load(d)
    ref.f("set_r_planet")()
    ref.prepare()
    ro, rs = ref.get("r_out"), ref.get("r_search")
    L = build_lists(d["pos"], d["mass"], rs, 0.5, 8, 64)
    n = len(d["mass"])
    epj = np.zeros(n, EPJ_DTYPE)
    epj["id_local"] = np.arange(n)
    epj["pos"] = d["pos"]
    epj["r_out"] = ro
    epj["r_search"] = rs
    epj["id"] = d["id"]
    epj["mass"] = d["mass"]
    epj["vel"] = d["vel"]
    epi = np.zeros(n, EPI_DTYPE)
    for k in EPI_DTYPE.names:
        epi[k] = epj[k]
    lib = H.load("ref")
    force = cleared_forces(n)
    for g in range(L["n_group"]):
        ii = L["i_idx"][L["i_off"][g]:L["i_off"][g + 1]]
        jj = L["j_idx"][L["j_off"][g]:L["j_off"][g + 1]]
        ss = L["s_idx"][L["s_off"][g]:L["s_off"][g + 1]]
        ei, ej, sj = (np.ascontiguousarray(x) for x in (epi[ii], epj[jj], L["spj"][ss]))
        f = cleared_forces(len(ii))
        lib.ref_epep(ei.ctypes.data_as(ctypes.c_void_p), len(ii), ej.ctypes.data_as(ctypes.c_void_p), len(jj),
                     f.ctypes.data_as(ctypes.c_void_p))
        lib.ref_epsp(ei.ctypes.data_as(ctypes.c_void_p), len(ii), sj.ctypes.data_as(ctypes.c_void_p), len(ss),
                     f.ctypes.data_as(ctypes.c_void_p))
        force[ii] = f
    np.savez_compressed(os.path.join(HERE, "soft_functor.npz"), params=P.vector(), epj=epj.view(np.uint8),
                        spj=L["spj"].view(np.uint8), force=force.view(np.uint8),
                        **{k: L[k] for k in ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx")})


def scalar_fixture():
    """Cutoff functions and Kepler's equation on a grid."""
    P = P3TParams(gamma=0.1)
    ref = H.CpuSystem("ref", P)
    lib = ref.lib
    r = np.linspace(0.0, 1.2, 241)[1:]
    W = np.array([lib.ref_cutoff_W(x, 1.0) for x in r])
    K = np.array([lib.ref_cutoff_K(x, 1.0) for x in r])
    dK = np.array([lib.ref_cutoff_dKdt(x, 1.0, 0.3) for x in r])
    consts = np.zeros(5)
    lib.ref_get_gamma_consts(consts.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    l = np.linspace(-3.0, 9.0, 97)
    e = np.array([0.0, 1e-4, 0.01, 0.1, 0.5, 0.79])
    U = np.array([[lib.ref_solve_kepler(a, b) for a in l] for b in e])
    np.savez_compressed(os.path.join(HERE, "scalars.npz"), r=r, W=W, K=K, dKdt=dK, gamma_consts=consts, l=l,
                        ecc=e, u=U, params=P.vector())


def step_fixture():
    """A 600-body disk (enlarged radii, so that it collides) through start-up
    and 4 tree steps: per-step state snapshots."""
    P = P3TParams()
    d = make_disk(600, 1e-9, 0.99, 1.01, ecc_hill=2.0, inc_hill=1.0, seed=13, f=150.0)
    ref = H.CpuSystem("ref", P)
    lf = H.tree_lists_fn(P)
    snaps = {}
    e0 = H.p3t_init(ref, d, lf)

    def snap(tag):
        for k in ("pos", "vel", "acc", "acc_d", "jerk_d", "phi", "phi_d", "dt", "acc0", "mass", "r_out",
                  "r_search"):
            snaps[f"{tag}_{k}"] = ref.get(k)
        for k in ("id", "id_cluster", "number", "n_cluster"):
            snaps[f"{tag}_{k}"] = ref.get(k)
        snaps[f"{tag}_pairs"] = ref.pairs()
        snaps[f"{tag}_energy"] = ref.energy()

    snap("init")
    ncol = 0
    for s in range(1, 5):
        out = H.p3t_step(ref, s, lf)
        snaps[f"s{s}_cols"] = out["cols"]
        snaps[f"s{s}_edisp"] = out["edisp"]
        ncol += len(out["cols"])
        snap(f"s{s}")
    np.savez_compressed(os.path.join(HERE, "p3t_steps.npz"), params=P.vector(), e0=e0, ncol=ncol,
                        **{f"disk_{k}": v for k, v in d.items()}, **snaps)
    return ncol


if __name__ == "__main__":
    H.build_oracle(with_ref=True)
    soft_functor_fixture()
    scalar_fixture()
    nc = step_fixture()
    print("fixtures written; collisions in the step fixture:", nc)
