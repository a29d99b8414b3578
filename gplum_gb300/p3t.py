"""The device-resident P3T step through the C ABI (include/gplum_p3t.h).

:class:`GpuSystem` exposes the phases of GPLUM's tree step
(src/main_p3t.cpp:423-717) on a particle system that stays in HBM, with the
same method names as the CPU checkers' harness, so one driver runs a
scenario on either.  Interaction lists come from the host tree
(gplum_gb300.tree) built on the current positions.
"""
import ctypes

import numpy as np

from . import _lib
from .soft import configure

VP = ctypes.c_void_p
# phases of p3t_step_phases_ms (include/gplum_p3t.h P3T_PH_*)
STEP_PHASES = ("kick1", "cluster", "hard", "tree_soft", "correct", "kick2", "energy", "merge", "remove", "reforce")


class LoopParams(ctypes.Structure):
    """p3t_loop_params_t"""
    _fields_ = [("theta", ctypes.c_double), ("n_leaf_limit", ctypes.c_int), ("n_group_limit", ctypes.c_int),
                ("reset_step", ctypes.c_int), ("r_max", ctypes.c_double), ("r_min", ctypes.c_double)]


class StepResult(ctypes.Structure):
    """p3t_step_result_t"""
    _fields_ = [("n_col", ctypes.c_int), ("n_removed", ctypes.c_int), ("n_body", ctypes.c_int),
                ("reforced", ctypes.c_int), ("n_clusters", ctypes.c_int), ("n_isolated", ctypes.c_int),
                ("energy", ctypes.c_double * 5), ("edisp", ctypes.c_double),
                ("edisp_hard", ctypes.c_double * 2)]


VEC_FIELDS = {"pos": 0, "vel": 1, "acc": 2, "acc_d": 3, "jerk_d": 4, "acc_s": 5, "jerk_s": 6}
SCALAR_FIELDS = {"phi": 10, "phi_d": 11, "phi_s": 12, "mass": 13, "r_out": 14, "r_search": 15, "dt": 16,
                 "acc0": 17, "time": 18, "r_planet": 19, "v_disp": 20, "r_out_inv": 21, "f": 22}
I64_FIELDS = {"id": 100, "id_cluster": 101}
I32_FIELDS = {"number": 102, "n_cluster": 103, "dead": 104, "merged": 105, "rank": 106, "id_min": 107,
              "id_max": 108}


class GpuSystem:
    kind = "gpu"

    def __init__(self, params, precision=0, trace_mode=0, cand_cap=64):
        self.lib = configure(params, precision, trace_mode, cand_cap)
        self.params = params
        self.cand_cap = cand_cap

    def _chk(self, st, what):
        _lib.check(st, what)

    def load(self, disk):
        a = [np.ascontiguousarray(disk[k], dtype=t) for k, t in
             (("id", np.int64), ("mass", np.float64), ("r_planet", np.float64), ("f", np.float64),
              ("pos", np.float64), ("vel", np.float64))]
        self._chk(self.lib.p3t_state_load(len(a[1]), *(x.ctypes.data_as(VP) for x in a)), "p3t_state_load")

    @property
    def n(self):
        return self.lib.p3t_state_n()

    def get(self, name):
        n = self.n
        if name in VEC_FIELDS:
            out, code = np.zeros((n, 3)), VEC_FIELDS[name]
        elif name in SCALAR_FIELDS:
            out, code = np.zeros(n), SCALAR_FIELDS[name]
        elif name in I64_FIELDS:
            out, code = np.zeros(n, np.int64), I64_FIELDS[name]
        else:
            out, code = np.zeros(n, np.int32), I32_FIELDS[name]
        self._chk(self.lib.p3t_state_get(code, out.ctypes.data_as(VP)), "p3t_state_get")
        return out

    def set(self, name, val):
        code = VEC_FIELDS.get(name, SCALAR_FIELDS.get(name))
        dt = np.float64
        if code is None and name in I64_FIELDS:
            code, dt = I64_FIELDS[name], np.int64
        elif code is None:
            code, dt = I32_FIELDS[name], np.int32
        val = np.ascontiguousarray(val, dtype=dt)
        self._chk(self.lib.p3t_state_set(code, val.ctypes.data_as(VP)), "p3t_state_set")

    def set_r_planet(self):
        self._chk(self.lib.p3t_set_r_planet(), "p3t_set_r_planet")

    def prepare(self):
        """setIDLocalAndMyrank (implicit: index order) + setCutoffRadii."""
        self._chk(self.lib.p3t_set_cutoff_radii(), "p3t_set_cutoff_radii")

    def soft_force(self, L):
        st = self.lib.p3t_state_soft(L["n_group"], *(L[k].ctypes.data_as(VP) for k in
                                                     ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx")),
                                     L["spj"].ctypes.data_as(VP), len(L["spj"]))
        self._chk(st, "p3t_state_soft")

    def correct(self, initial):
        self._chk(self.lib.p3t_correct(1 if initial else 0), "p3t_correct")

    def neighbor_ids_local(self, i):
        # the library widens its neighbour table past cand_cap when a body needs it
        cap = max(self.cand_cap, 1 << 14)
        out = np.zeros(cap, np.int32)
        m = self.lib.p3t_neighbor_list(i, out.ctypes.data_as(VP), cap)
        return out[:max(m, 0)]

    def pairs(self):
        """(i, j) with i < j, j a neighbour of i (NeighborList::pair_list),
        ordered by i and then j."""
        m = self.lib.p3t_neighbor_pairs(None, 0)
        if m < 0:
            raise RuntimeError(f"p3t_neighbor_pairs failed with status {m}")
        out = np.zeros((max(m, 1), 2), np.int32)
        m2 = self.lib.p3t_neighbor_pairs(out.ctypes.data_as(VP), m)
        if m2 != m:
            raise RuntimeError(f"p3t_neighbor_pairs returned {m2}, expected {m}")
        return out[:m]

    def cluster(self):
        self._chk(self.lib.p3t_cluster_label(), "p3t_cluster_label")

    def cluster_lists(self):
        nc = ctypes.c_int(0)
        self._chk(self.lib.p3t_cluster_lists(ctypes.byref(nc), None, None), "p3t_cluster_lists")
        off = np.zeros(nc.value + 1, np.int32)
        mem = np.zeros(max(1, self.n), np.int32)
        self._chk(self.lib.p3t_cluster_lists(ctypes.byref(nc), off.ctypes.data_as(VP), mem.ctypes.data_as(VP)),
                  "p3t_cluster_lists")
        return off, mem[:off[-1]]

    def kick(self):
        self._chk(self.lib.p3t_kick(), "p3t_kick")

    def hard(self, istep, col_cap=4096):
        cols = np.zeros(2 * col_cap, np.int64)
        ed = np.zeros(2)
        nc = self.lib.p3t_hard(istep, col_cap, cols.ctypes.data_as(VP), ed.ctypes.data_as(VP))
        if nc < 0:
            bits = _lib.status_bits(nc)
            raise RuntimeError(f"p3t_hard failed: kernel status bits {bits}" if bits else
                               f"p3t_hard failed with status {nc}")
        return cols[:2 * min(nc, col_cap)].reshape(-1, 2), ed

    def set_fragmentation(self, a_frag, n_frag=10, m_min=9.426627927538057e-12, seed=0):
        """KOMINAMI fragmentation of the collision outcome (a_frag = 0: off)."""
        self._chk(self.lib.p3t_set_fragmentation(a_frag, n_frag, m_min, seed), "p3t_set_fragmentation")

    def id_next(self):
        return int(self.lib.p3t_id_next())

    def write_snapshot(self, path, binary, header, async_write=False):
        """The state to a GPLUM snapshot file (snapNNNNNN.dat ASCII or the
        snap_tmp.dat binary restart); with async_write the file is written by
        a host thread while later phases run (wait_snapshot joins it)."""
        h = header._c()
        self._chk(self.lib.p3t_snapshot_write(str(path).encode(), int(binary), ctypes.byref(h),
                                              1 if async_write else 0), "p3t_snapshot_write")

    def wait_snapshot(self):
        self._chk(self.lib.p3t_snapshot_wait(), "p3t_snapshot_wait")

    def read_snapshot(self, path, binary):
        """Loads a GPLUM snapshot file into the state (GPLUM's start-up read);
        returns its header."""
        from .snapshot import Header, _Header
        h = _Header()
        n = self.lib.p3t_snapshot_read(str(path).encode(), int(binary), ctypes.byref(h))
        if n < 0:
            raise RuntimeError(f"p3t_snapshot_read failed with status {n}")
        return Header._from(h)

    def tree_soft(self):
        """Device octree + interaction lists from the current state, then the
        soft force (replaces a host build_lists + soft_force pair)."""
        P = self.params
        self._chk(self.lib.p3t_state_tree_soft(P.theta, P.n_leaf_limit, P.n_group_limit), "p3t_state_tree_soft")

    def tree_lists(self, build=True):
        """The resident lists as a dict in build_lists' layout (optionally
        building them on the device first)."""
        from .layout import SPJ_DTYPE
        P = self.params
        if build:
            self._chk(self.lib.p3t_state_tree(P.theta, P.n_leaf_limit, P.n_group_limit), "p3t_state_tree")
        c = np.zeros(5, np.int64)
        self._chk(self.lib.p3t_tree_lists_counts(c.ctypes.data_as(VP)), "p3t_tree_lists_counts")
        ng, ni, nj, ns, nn = (int(x) for x in c)
        out = dict(n_group=ng, i_off=np.zeros(ng + 1, np.int32), i_idx=np.zeros(ni, np.int32),
                   j_off=np.zeros(ng + 1, np.int32), j_idx=np.zeros(nj, np.int32),
                   s_off=np.zeros(ng + 1, np.int32), s_idx=np.zeros(ns, np.int32), spj=np.zeros(nn, SPJ_DTYPE))
        self._chk(self.lib.p3t_tree_lists_get(*(out[k].ctypes.data_as(VP) for k in
                                                ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx", "spj"))),
                  "p3t_tree_lists_get")
        return out

    def hard_costs(self):
        """(block steps, pair sweeps) of each cluster of the last hard launch."""
        nc = len(self.cluster_lists()[0]) - 1
        out = np.zeros(2 * max(nc, 1), np.int64)
        self._chk(self.lib.p3t_hard_costs(out.ctypes.data_as(VP), nc), "p3t_hard_costs")
        return out[:2 * nc].reshape(-1, 2)

    def hard_times(self):
        """(start, end) of each cluster's integration, device global timer (ns)."""
        nc = len(self.cluster_lists()[0]) - 1
        out = np.zeros(2 * max(nc, 1), np.int64)
        self._chk(self.lib.p3t_hard_times(out.ctypes.data_as(VP), nc), "p3t_hard_times")
        return out[:2 * nc].reshape(-1, 2)

    def cluster_features(self):
        """The learned scheduler's four features of each current cluster."""
        nc = len(self.cluster_lists()[0]) - 1
        out = np.zeros((max(nc, 1), 4), np.float32)
        self._chk(self.lib.p3t_cluster_features(out.ctypes.data_as(VP), nc), "p3t_cluster_features")
        return out[:nc]

    def energy(self):
        out = np.zeros(5)
        self._chk(self.lib.p3t_energy(out.ctypes.data_as(VP)), "p3t_energy")
        return out

    def merge(self, n_col):
        e = ctypes.c_double(0.0)
        self._chk(self.lib.p3t_merge(ctypes.byref(e)), "p3t_merge")
        return e.value

    def remove(self, r_max, r_min):
        """removeParticlesOutOfBoundary: (bodies removed, energy they took)."""
        e = ctypes.c_double(0.0)
        n = self.lib.p3t_remove_out_of_boundary(r_max, r_min, ctypes.byref(e))
        if n < 0:
            raise RuntimeError(f"p3t_remove_out_of_boundary failed with status {n}")
        return n, e.value

    # the whole tree step as one native call (include/gplum_p3t.h p3t_tree_step)
    def startup(self, reset_step=1024, r_max=40.0, r_min=0.1):
        """Cutoff radii and two passes of soft force + correctForceLongInitial
        (src/main_p3t.cpp:289-364); returns the initial energy."""
        P = self.params
        lp = LoopParams(P.theta, P.n_leaf_limit, P.n_group_limit, reset_step, r_max, r_min)
        e = np.zeros(5)
        self._chk(self.lib.p3t_startup(ctypes.byref(lp), e.ctypes.data_as(VP)), "p3t_startup")
        return e

    def tree_step(self, istep):
        """One tree step (src/main_p3t.cpp:423-717) in the library; returns
        the p3t_step_result_t fields as a dict."""
        res = StepResult()
        self._chk(self.lib.p3t_tree_step(istep, ctypes.byref(res)), "p3t_tree_step")
        return {"n_col": res.n_col, "n_removed": res.n_removed, "n_body": res.n_body, "reforced": res.reforced,
                "n_clusters": res.n_clusters, "n_isolated": res.n_isolated, "energy": np.array(res.energy[:]),
                "edisp": res.edisp, "edisp_hard": np.array(res.edisp_hard[:])}

    def step_phases_ms(self):
        """Device time of each phase of the last tree_step (CUDA events)."""
        ms = np.zeros(len(STEP_PHASES), np.float32)
        self._chk(self.lib.p3t_step_phases_ms(ms.ctypes.data_as(VP)), "p3t_step_phases_ms")
        return dict(zip(STEP_PHASES, ms.astype(float).tolist()))

    def collisions(self):
        """(impactor id, target id) of the last hard part's collisions, in
        collision-list order."""
        from .collisions import records
        return np.array([(r.id_imp, r.id_tar) for r in records(self.lib)], np.int64).reshape(-1, 2)

    def put_fpgrav(self, records, id_next=-1):
        """The state from an array of GPLUM FPGrav records (layout.FPGRAV_DTYPE)."""
        self._chk(self.lib.p3t_state_put_fpgrav(len(records), records.ctypes.data_as(VP), int(id_next)),
                  "p3t_state_put_fpgrav")

    def get_fpgrav(self, out=None):
        """The state as an array of GPLUM FPGrav records (into `out` when it
        is large enough)."""
        from .layout import FPGRAV_DTYPE
        n = self.n
        if out is None or len(out) < n:
            out = np.zeros(n, FPGRAV_DTYPE)
        m = self.lib.p3t_state_get_fpgrav(out.ctypes.data_as(VP), len(out))
        if m < 0:
            raise RuntimeError(f"p3t_state_get_fpgrav failed with status {m}")
        return out[:m]

    def hard_launch_stats(self):
        """The last cluster launch: dict of its device time (ms), the pair
        terms it evaluated in predicted/corrected passes and in full-force
        passes (counted by the bundle form), and sums over its clusters
        (pair sweeps, n(n-1) x block steps, active members over block steps,
        largest block-step count, member predictions)."""
        ms = ctypes.c_double(0.0)
        p = np.zeros(3, np.int64)
        sm = np.zeros(5)
        self._chk(self.lib.p3t_hard_launch_stats(ctypes.byref(ms), p.ctypes.data_as(VP), sm.ctypes.data_as(VP)),
                  "p3t_hard_launch_stats")
        return {"ms": ms.value, "live_pc": int(p[0]), "live_full": int(p[1]), "counted": bool(p[2]),
                "sweeps": float(sm[0]), "coll_pairs": float(sm[1]), "active": float(sm[2]),
                "max_block_steps": int(sm[3]), "predictions": float(sm[4])}

    def counts(self):
        a, b = ctypes.c_int(), ctypes.c_int()
        self._chk(self.lib.p3t_neighbor_counts(ctypes.byref(a), ctypes.byref(b)), "p3t_neighbor_counts")
        return a.value, b.value

    # interface of the checkers' harness (oracle/harness.py)
    def f(self, name):
        if name == "set_r_planet":
            return self.set_r_planet
        if name == "set_id_local":
            return lambda: None
        if name == "n_cluster":
            return lambda: len(self.cluster_lists()[0]) - 1
        if name == "n_isolated":
            return lambda: int((self.get("number") == 0).sum())
        raise AttributeError(name)
