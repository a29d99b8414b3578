"""Snapshots of the device state: the device writer against the host writer
on the same fields (byte for byte, also when written asynchronously while
later steps run), and a restart from the binary file that continues exactly
as the run that wrote it (both recompute the cutoff radii and the forces
after the write, as GPLUM's restart does)."""
import numpy as np
import pytest

from gplum_gb300 import run as R
from gplum_gb300 import snapshot
from gplum_gb300.disk import P3TParams, make_disk
from gplum_gb300.p3t import GpuSystem

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "acc", "acc_d", "jerk_d", "acc_s", "jerk_s", "phi", "phi_d", "phi_s", "mass", "r_planet",
          "f", "r_out", "r_search", "r_out_inv", "v_disp", "time", "dt", "acc0", "id", "id_cluster", "number",
          "rank", "id_max", "id_min", "n_cluster", "dead", "merged")
CARRIED = ("pos", "vel", "acc_d", "jerk_d", "acc_s", "jerk_s", "phi_d", "phi_s", "mass", "r_planet", "f", "dt",
           "acc0", "id", "id_cluster", "v_disp")


def state(g):
    return {k: g.get(k) for k in FIELDS}


def continue_run(g, first, last):
    g.prepare()
    g.tree_soft()
    g.correct(False)
    for st in range(first, last + 1):
        R.step(g, st)


def test_device_snapshots_and_restart(gpu, tmp_path):
    P = P3TParams()
    disk = make_disk(600, 1e-9, 0.99, 1.01, ecc_hill=2.0, inc_hill=1.0, seed=21, f=150.0)
    g = GpuSystem(P)
    e0 = R.startup(g, disk)
    ncol = 0
    for st in (1, 2):
        cols, e, _ = R.step(g, st)
        ncol += len(cols)
    hdr = snapshot.Header(time=2 * P.dt_tree, id_next=g.id_next(), e_init=snapshot.energy7(e0),
                          e_now=snapshot.energy7(e, 1e-15))
    s2 = state(g)
    binp, txtp = tmp_path / "snap_tmp.dat", tmp_path / "snap000001.dat"
    g.write_snapshot(binp, 1, hdr)
    g.write_snapshot(txtp, 0, hdr, async_write=True)  # formatted while the next steps run
    continue_run(g, 3, 5)
    g.wait_snapshot()
    final_a = state(g)
    # the device files equal the host writer's on the state at the write
    for path, binary in ((binp, 1), (txtp, 0)):
        ref = tmp_path / f"host_{binary}.dat"
        src = {k: s2[k] for k in FIELDS} if binary else {k: s2[k] for k in snapshot.ASCII_FIELDS}
        snapshot.write_host(ref, binary, hdr, src)
        assert path.read_bytes() == ref.read_bytes(), path
    # restart from the binary file: the carried fields come back bit for bit
    h = g.read_snapshot(binp, 1)
    assert h.n_body == len(s2["id"]) and h.time == hdr.time and g.id_next() == hdr.id_next
    for k in CARRIED:
        np.testing.assert_array_equal(g.get(k), s2[k], err_msg=k)
    np.testing.assert_array_equal(g.get("time"), np.full(len(s2["id"]), hdr.time))
    assert not g.get("number").any() and not g.get("dead").any()
    continue_run(g, 3, 5)
    final_b = state(g)
    for k in FIELDS:
        np.testing.assert_array_equal(final_b[k], final_a[k], err_msg=k)
    # an ASCII snapshot starts a run like an initial-condition file
    h = g.read_snapshot(txtp, 0)
    assert h.n_body == len(s2["id"])
    np.testing.assert_array_equal(g.get("id"), s2["id"])
