"""The whole tree step as one native call (p3t_startup / p3t_tree_step) and
the FPGrav record exchange, on the GPU:

* p3t_tree_step equals the same phases called one by one through the C ABI
  (gplum_gb300.run.step), bit for bit, and tracks the CPU oracle's step;
* FPGrav records (GPLUM's ParticleSystem<FPGrav> element) go to the device
  and back unchanged, and a step taken after the round trip equals one taken
  without it;
* the step's phase times come from the GPU (positive, summing to the step),
  the launch counter advances, and the hard launch reports its time and the
  pair terms it evaluated.
"""
import numpy as np
import pytest

from gplum_gb300.disk import P3TParams, make_disk
from gplum_gb300.layout import FPGRAV_DTYPE
from gplum_gb300.p3t import STEP_PHASES, GpuSystem
from oracle import harness as H
from tests.common import rel_err

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "acc", "acc_d", "jerk_d", "acc_s", "jerk_s", "phi", "phi_d", "dt", "time", "mass", "id",
          "id_cluster", "number")


def _disk(n=3000, seed=21):
    # radii enlarged (f = 150, as GPLUM's increase factor) so that bodies collide every few steps
    return make_disk(n, 1e-9, 0.97, 1.03, ecc_hill=4.0, inc_hill=2.0, seed=seed, f=150.0)


def _state(g):
    return {k: g.get(k) for k in FIELDS}


def test_native_step_equals_phase_calls(gpu):
    from gplum_gb300 import run

    P = P3TParams()
    d = _disk()
    a = GpuSystem(P)
    a.load(d)
    a.set_r_planet()
    e0a = a.startup()
    sa = []
    for istep in range(1, 6):
        r = a.tree_step(istep)
        sa.append((_state(a), r["n_col"], r["energy"].copy(), r["edisp"], a.collisions()))
    b = GpuSystem(P)
    e0b = run.startup(b, d)
    np.testing.assert_array_equal(e0a, e0b)
    for istep in range(1, 6):
        cols, e, ed = run.step(b, istep)
        st, ncol, ea, eda, ca = sa[istep - 1]
        assert ncol == len(cols)
        np.testing.assert_array_equal(ca, cols)
        np.testing.assert_array_equal(ea, e)
        assert eda == ed
        for k, v in _state(b).items():
            np.testing.assert_array_equal(st[k], v, err_msg=f"step {istep} {k}")
    assert sum(s[1] for s in sa) > 0, "the case should include collisions"


def test_native_step_tracks_the_oracle(gpu):
    P = P3TParams()
    d = make_disk(1000, 1e-9, 0.98, 1.02, ecc_hill=4.0, inc_hill=2.0, seed=9)
    orc = H.CpuSystem("orc", P)
    lf = H.tree_lists_fn(P)
    H.p3t_init(orc, d, lf)
    g = GpuSystem(P)
    g.load(d)
    g.set_r_planet()
    g.startup()
    for istep in range(1, 4):
        a = H.p3t_step(orc, istep, lf)
        r = g.tree_step(istep)
        np.testing.assert_array_equal(a["cols"], g.collisions())
        assert g.n == orc.n
        np.testing.assert_array_equal(g.get("id"), orc.get("id"))
        assert rel_err(g.get("pos"), orc.get("pos")).max() < 1e-10
        assert abs(r["energy"][0] - a["energy"][0]) <= 1e-12 * abs(a["energy"][0])


def test_fpgrav_round_trip(gpu):
    P = P3TParams()
    d = _disk(2000, seed=5)
    g = GpuSystem(P)
    g.load(d)
    g.set_r_planet()
    g.startup()
    g.tree_step(1)
    rec = g.get_fpgrav()
    assert rec.dtype == FPGRAV_DTYPE and len(rec) == g.n
    np.testing.assert_array_equal(rec["pos"], g.get("pos"))
    np.testing.assert_array_equal(rec["id"], g.get("id"))
    np.testing.assert_array_equal(rec["id_local"], np.arange(g.n))
    assert (rec["in_domain"] == 1).all()
    before = _state(g)
    g.put_fpgrav(rec.copy())
    for k, v in _state(g).items():
        np.testing.assert_array_equal(before[k], v, err_msg=k)
    assert g.get_fpgrav().tobytes() == rec.tobytes()
    # a step after the round trip equals a step without it (the same run twice)
    out = []
    for trip in (False, True):
        g.load(d)
        g.set_r_planet()
        g.startup()
        g.tree_step(1)
        if trip:
            g.put_fpgrav(g.get_fpgrav())
        g.tree_step(2)
        out.append(_state(g))
    for k in FIELDS:
        np.testing.assert_array_equal(out[0][k], out[1][k], err_msg=k)


def test_phase_times_launch_count_and_hard_stats(gpu):
    P = P3TParams()
    g = GpuSystem(P)
    g.load(_disk(3000, seed=7))
    g.set_r_planet()
    g.startup()
    c0 = g.lib.p3t_launch_count()
    g.tree_step(1)
    c1 = g.lib.p3t_launch_count()
    assert c1 - c0 > 20
    ph = g.step_phases_ms()
    assert list(ph) == list(STEP_PHASES)
    assert all(v >= 0.0 for v in ph.values()) and ph["hard"] > 0.0 and ph["tree_soft"] > 0.0
    h = g.hard_launch_stats()
    assert h["counted"] and h["ms"] > 0.0 and h["live_pc"] > 0 and h["live_full"] > 0
    assert h["ms"] <= ph["hard"] + 1e-3
    assert h["sweeps"] > 0 and h["active"] > 0 and h["max_block_steps"] >= 1
    # every evaluated predicted/corrected term is one of GPLUM's 3 n_act n sweeps
    assert h["live_pc"] <= 3 * h["sweeps"]
