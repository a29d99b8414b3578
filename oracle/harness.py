"""ctypes harness over the two CPU checkers.  TEST INFRASTRUCTURE ONLY.

``CpuSystem("orc")`` drives the CPU restatement (oracle/_build/libp3t_oracle.so,
built by oracle/Makefile on any machine); ``CpuSystem("ref")`` drives GPLUM's
own headers compiled against the PS shim (oracle/_ref/libgplum_ref.so, only
where the reference tree was present at build time).  Both expose the same
surface, so a test runs one scenario through either and compares.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline legs import
this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libp3t_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libgplum_ref.so")
REF_KOM_SO = os.path.join(HERE, "_ref", "libgplum_ref_kominami.so")
# GPLUM's src/ directory, for the reference build (from the environment; the
# build recipe in __graft_entry__.py sets it where the reference tree exists)
REF_SRC = os.environ.get("GPLUM_REF_SRC", "")

F64P = ctypes.POINTER(ctypes.c_double)
I32P = ctypes.POINTER(ctypes.c_int)
I64P = ctypes.POINTER(ctypes.c_longlong)
VP = ctypes.c_void_p

# field codes of *_get_f64 / *_get_i64
VEC_FIELDS = {"pos": 0, "vel": 1, "acc": 2, "acc_d": 3, "jerk_d": 4, "acc_s": 5, "jerk_s": 6}
SCALAR_FIELDS = {"phi": 10, "phi_d": 11, "phi_s": 12, "mass": 13, "r_out": 14, "r_search": 15,
                 "dt": 16, "acc0": 17, "time": 18, "r_planet": 19, "v_disp": 20, "r_out_inv": 21, "f": 22}
INT_FIELDS = {"id": 0, "id_cluster": 1, "number": 2, "n_cluster": 3, "dead": 4, "merged": 5,
              "rank": 6, "id_min": 7, "id_max": 8}


def build_oracle(with_ref=None):
    """Compiles the restatement (always) and the reference build (when the
    reference tree exists).  Quick: two translation units."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    ref_src = os.environ.get("GPLUM_REF_SRC", REF_SRC)
    if with_ref is None:
        with_ref = bool(ref_src) and os.path.isdir(ref_src)
    if with_ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_SRC={ref_src}"], check=True)


def ref_available():
    return os.path.exists(REF_SO)


def ref_source_dir():
    """GPLUM's src/ directory the reference build was compiled from (None
    where there is no reference build)."""
    p = os.path.join(HERE, "_ref", "ref_src.txt")
    if not os.path.exists(p):
        return None
    d = open(p).read().strip()
    return d if d and os.path.isdir(d) else None


def _ptr(a, t):
    return a.ctypes.data_as(t)


_LIBS = {}


def load(kind):
    """kind: "orc" (restatement), "ref" (reference build), "ref_kominami"
    (reference build with the KOMINAMI fragmentation model; symbols ref_*)."""
    if kind in _LIBS:
        return _LIBS[kind]
    path = {"orc": ORACLE_SO, "ref": REF_SO, "ref_kominami": REF_KOM_SO}[kind]
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    lib = ctypes.CDLL(path)
    p = kind.split("_")[0] + "_"
    for name, res in [("cutoff_W", ctypes.c_double), ("cutoff_K", ctypes.c_double),
                      ("cutoff_dKdt", ctypes.c_double), ("solve_kepler", ctypes.c_double),
                      ("n", ctypes.c_int), ("n_pairs", ctypes.c_int), ("hard", ctypes.c_int),
                      ("n_cluster", ctypes.c_int), ("n_isolated", ctypes.c_int),
                      ("n_list_size", ctypes.c_int), ("n_ngb_tot", ctypes.c_int),
                      ("n_with_ngb", ctypes.c_int)]:
        getattr(lib, p + name).restype = res
    getattr(lib, p + "cutoff_W").argtypes = [ctypes.c_double, ctypes.c_double]
    getattr(lib, p + "cutoff_K").argtypes = [ctypes.c_double, ctypes.c_double]
    getattr(lib, p + "cutoff_dKdt").argtypes = [ctypes.c_double] * 3
    getattr(lib, p + "solve_kepler").argtypes = [ctypes.c_double] * 2
    _LIBS[kind] = lib
    return lib


class CpuSystem:
    """One particle system inside a checker library (process-global state)."""

    def __init__(self, kind, params):
        self.kind = kind
        self.lib = load(kind)
        self.params = params
        self.f("set_params")(_ptr(np.ascontiguousarray(params.vector()), F64P))

    def f(self, name):
        return getattr(self.lib, f"{self.kind}_{name}")

    def set_fragmentation(self, a_frag, n_frag=10, m_min=9.426627927538057e-12, seed=0):
        """KOMINAMI fragmentation in the restatement, with the keyed phase
        draw the device uses (a_frag = 0: off)."""
        assert self.kind == "orc"
        self.lib.orc_set_frag(ctypes.c_double(a_frag), ctypes.c_int(n_frag), ctypes.c_double(m_min), ctypes.c_int(0),
                              ctypes.c_ulonglong(seed))

    def remove(self, r_max, r_min):
        """removeParticlesOutOfBoundary: (bodies removed, energy they took)."""
        e = ctypes.c_double(0.0)
        fn = self.f("remove")
        fn.restype = ctypes.c_int
        n = fn(ctypes.c_double(r_max), ctypes.c_double(r_min), ctypes.byref(e))
        return n, e.value

    def id_next(self):
        self.lib.orc_id_next.restype = ctypes.c_longlong
        return int(self.lib.orc_id_next())

    def load(self, disk):
        n = len(disk["mass"])
        self._keep = [np.ascontiguousarray(disk[k]) for k in ("id", "mass", "r_planet", "f", "pos", "vel")]
        idv, m, rp, f, pos, vel = self._keep
        self.f("load")(ctypes.c_int(n), _ptr(idv.astype(np.int64), I64P), _ptr(m, F64P), _ptr(rp, F64P),
                       _ptr(f, F64P), _ptr(pos, F64P), _ptr(vel, F64P))

    @property
    def n(self):
        return self.f("n")()

    def get(self, name):
        n = self.n
        if name in VEC_FIELDS:
            out = np.zeros((n, 3))
            self.f("get_f64")(VEC_FIELDS[name], _ptr(out, F64P))
        elif name in SCALAR_FIELDS:
            out = np.zeros(n)
            self.f("get_f64")(SCALAR_FIELDS[name], _ptr(out, F64P))
        else:
            out = np.zeros(n, np.int64)
            self.f("get_i64")(INT_FIELDS[name], _ptr(out, I64P))
        return out

    def set(self, name, val):
        val = np.ascontiguousarray(val, dtype=np.float64)
        code = VEC_FIELDS.get(name, SCALAR_FIELDS.get(name))
        self.f("set_f64")(code, _ptr(val, F64P))

    def prepare(self):
        """setIDLocalAndMyrank + setCutoffRadii."""
        self.f("set_id_local")()
        self.f("set_cutoff_radii")()

    def soft_force(self, lists):
        self.f("soft_force")(ctypes.c_int(lists["n_group"]), _ptr(lists["i_off"], I32P),
                             _ptr(lists["i_idx"], I32P), _ptr(lists["j_off"], I32P),
                             _ptr(lists["j_idx"], I32P), _ptr(lists["s_off"], I32P),
                             _ptr(lists["s_idx"], I32P), lists["spj"].ctypes.data_as(VP))

    def correct(self, initial):
        self.f("correct")(ctypes.c_int(1 if initial else 0))

    def pairs(self):
        k = self.f("n_pairs")()
        out = np.zeros(2 * k, np.int32)
        self.f("get_pairs")(_ptr(out, I32P))
        return out.reshape(-1, 2)

    def neighbor_ids(self, i):
        k = self.f("n_list_size")(ctypes.c_int(i))
        out = np.zeros(k, np.int64)
        self.f("n_list")(ctypes.c_int(i), _ptr(out, I64P))
        return out

    def cluster(self):
        self.f("cluster")()

    def kick(self):
        self.f("kick")()

    def hard(self, istep):
        cols = np.zeros(2 * 4096, np.int64)
        ed = np.zeros(2)
        nc = self.f("hard")(ctypes.c_int(istep), _ptr(cols, I64P), ctypes.c_int(4096), _ptr(ed, F64P))
        if nc < 0:
            raise RuntimeError("hard part lost particles")
        return cols[:2 * nc].reshape(-1, 2), ed

    def energy(self):
        out = np.zeros(5)
        self.f("energy")(_ptr(out, F64P))
        return out

    def merge(self, n_col):
        e = ctypes.c_double(0.0)
        self.f("merge")(ctypes.c_int(n_col), ctypes.byref(e))
        return e.value


def p3t_init(sysm, disk, lists_fn):
    """GPLUM's start-up (src/main_p3t.cpp:289-364): radii, then two passes of
    soft force + correctForceLongInitial (USE_RE_SEARCH_NEIGHBOR)."""
    sysm.load(disk)
    sysm.f("set_r_planet")()
    sysm.prepare()
    for _ in range(2):
        sysm.soft_force(lists_fn(sysm))
        sysm.correct(True)
    return sysm.energy()


def p3t_step(sysm, istep, lists_fn, reset_step=1024, clock=None):
    """One tree step (src/main_p3t.cpp:423-717) on a single rank: kick,
    clusters, hard part, soft force + correction, kick, energy, merge,
    re-force after collisions.  Returns a dict of what the step produced.
    With `clock` a dict, adds each phase's wall time (seconds) under GPLUM's
    CALC_WTIME names (src/time.h, src/main_p3t.cpp:437-710): calc_soft_force
    (kicks, tree + lists, soft force, energy, merge, radii),
    create_cluster, calc_hard_force, neighbor_search (correction)."""
    import time

    def timed(name, fn, *a):
        t0 = time.perf_counter()
        r = fn(*a)
        if clock is not None:
            clock[name] = clock.get(name, 0.0) + time.perf_counter() - t0
        return r

    timed("calc_soft_force", sysm.kick)
    timed("create_cluster", sysm.cluster)
    cols, edisp = timed("calc_hard_force", sysm.hard, istep)
    n_clusters = sysm.f("n_cluster")()
    n_iso = sysm.f("n_isolated")()
    sysm.f("set_id_local")()
    timed("calc_soft_force", lambda: sysm.soft_force(lists_fn(sysm)))
    timed("neighbor_search", sysm.correct, False)
    timed("calc_soft_force", sysm.kick)
    e = timed("calc_soft_force", sysm.energy)
    out = dict(cols=cols, edisp=edisp, n_clusters=n_clusters, n_iso=n_iso, energy=e)
    n_col = len(cols)
    if n_col:
        out["edisp_merge"] = timed("calc_soft_force", sysm.merge, n_col)
    if n_col or istep % reset_step == reset_step - 1:
        timed("calc_soft_force", sysm.prepare)
        timed("calc_soft_force", lambda: sysm.soft_force(lists_fn(sysm)))
        timed("neighbor_search", sysm.correct, True)
        out["energy"] = timed("calc_soft_force", sysm.energy)
    return out


def tree_lists_fn(params):
    """Interaction lists from the package's host tree for a checker system."""
    from gplum_gb300.tree import build_lists

    def fn(sysm):
        return build_lists(sysm.get("pos"), sysm.get("mass"), sysm.get("r_search"), params.theta,
                           params.n_leaf_limit, params.n_group_limit)
    return fn


# One collision in isolation (orc_collide_unit / ref_collide_unit): 26 doubles
# per FPHard record, in this order.
UNIT_FIELDS = ("x", "y", "z", "vx", "vy", "vz", "mass", "r_planet", "f", "r_out", "r_out_inv", "r_search",
               "v_disp", "time", "time_c", "dt", "phi", "phi_d", "phi_s", "acc0", "id", "id_cluster",
               "number", "dead", "merged", "spare")


def collide_unit(kind, params, frag, records, twins, imp, tar, id_next=0, seed=12345):
    """Runs one collision through the restatement ("orc", fragment phase
    from drand48 seeded with `seed`) or a reference build ("ref" /
    "ref_kominami", srand48(seed) first).  frag = (a_frag, N_frag, m_min).
    Returns (records after, n_frag, edisp[2], id_next after)."""
    lib = load(kind)
    pre = kind.split("_")[0] + "_"
    getattr(lib, pre + "set_params")(_ptr(np.ascontiguousarray(params.vector()), F64P))
    a_frag, n_frag, m_min = frag
    if kind == "orc":
        lib.orc_set_frag(ctypes.c_double(a_frag), ctypes.c_int(n_frag), ctypes.c_double(m_min), ctypes.c_int(1),
                         ctypes.c_ulonglong(seed))
    else:
        lib.ref_set_frag(ctypes.c_double(a_frag), ctypes.c_int(n_frag), ctypes.c_double(m_min))
        lib.ref_srand48(ctypes.c_long(seed))
    rec = np.ascontiguousarray(records, np.float64)
    n = len(rec)
    tw = np.ascontiguousarray(np.array(twins, np.int32).reshape(-1, 2))
    cap = n + 64
    out = np.zeros((cap, 26))
    ed = np.zeros(2)
    idn = ctypes.c_longlong(id_next)
    fn = getattr(lib, pre + "collide_unit")
    fn.restype = ctypes.c_int
    try:
        nf = fn(ctypes.c_int(n), _ptr(rec, F64P), ctypes.c_int(len(tw)), _ptr(tw, I32P), ctypes.c_int(imp),
                ctypes.c_int(tar), ctypes.byref(idn), _ptr(out, F64P), ctypes.c_int(cap), _ptr(ed, F64P))
    finally:  # back to perfect accretion for whatever runs next in this process
        if kind == "orc":
            lib.orc_set_frag(ctypes.c_double(0.0), ctypes.c_int(10), ctypes.c_double(9.426627927538057e-12),
                             ctypes.c_int(0), ctypes.c_ulonglong(0))
        else:
            lib.ref_set_frag(ctypes.c_double(0.0), ctypes.c_int(10), ctypes.c_double(9.426627927538057e-12))
    return out[:n + nf], nf, ed, idn.value
