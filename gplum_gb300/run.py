"""The P3T time loop on the device: GPLUM's main loop (src/main_p3t.cpp:
289-760) without its file output, on a GpuSystem whose tree, lists and every
phase of the step stay on the GPU.

    python -m gplum_gb300.run --steps 1000
    python -m gplum_gb300.run --workload embryos --a-frag 0.5 --schedule size --timing --steps 100
    python -m gplum_gb300.run --steps 1000 --output-dir out --snap-every 100 --snap-tmp-every 100
    python -m gplum_gb300.run --steps 2000 --output-dir out --restart

integrates the 3000-body disk (0.95-1.05 AU, m = 1e-9, rms e = 2 h,
rms i = h, dt_tree = 2^-7), or the embryo disk (1,048,576 planetesimals
plus four 0.1 Earth-mass embryos, KOMINAMI fragments with --a-frag), with
the hard queue in the learned or the size order, and prints the relative
energy error
(Energy::calcEnergyError, src/energy.h:65-67: (E - E_init - E_dissipated) /
E_init, where the dissipated energy sums the hard part's collisions, the
merges and the bodies removed outside [r_min, r_max],
src/main_p3t.cpp:539,641,645).
"""
import argparse
import json
import time

import numpy as np


def startup(g, disk):
    """src/main_p3t.cpp:289-364: radii, then two passes of device tree + soft
    force + correctForceLongInitial; returns the initial energy."""
    g.load(disk)
    g.set_r_planet()
    g.prepare()
    for _ in range(2):
        g.tree_soft()
        g.correct(True)
    return g.energy()


def step(g, istep, reset_step=1024, r_max=40.0, r_min=0.1, clock=None, stats=None):
    """One tree step (src/main_p3t.cpp:423-717; r_max and r_min as in
    parameter.dat, defaults src/read.h:111-112).  Returns (collision pairs,
    energy after the step, energy dissipated in this step).  With `clock` a
    dict, adds the synchronised wall time of each phase to it; with `stats` a
    list, appends the step's cluster counts after the hard part."""

    def timed(name, fn):
        if clock is None:
            return fn()
        g.lib.p3t_synchronize()
        t0 = time.perf_counter()
        r = fn()
        g.lib.p3t_synchronize()
        clock[name] = clock.get(name, 0.0) + time.perf_counter() - t0
        return r

    timed("kick", g.kick)
    timed("cluster", g.cluster)
    cols, ed = timed("hard", lambda: g.hard(istep))
    if stats is not None:
        stats.append(dict(step=istep, **cluster_stats(g)))
    edisp = float(ed[0])
    timed("tree_soft", g.tree_soft)
    timed("correct", lambda: g.correct(False))
    timed("kick", g.kick)
    e = timed("energy", g.energy)
    if len(cols):
        edisp += timed("merge", lambda: g.merge(len(cols)))
    n_rem, e_rem = timed("remove", lambda: g.remove(r_max, r_min))
    edisp += e_rem
    if len(cols) or n_rem or istep % reset_step == reset_step - 1:
        timed("radii", g.prepare)
        timed("tree_soft", g.tree_soft)
        timed("correct", lambda: g.correct(True))
        e = timed("energy", g.energy)
    return cols, e, edisp


def cluster_stats(g):
    """The hard system's counts as GPLUM logs them at snapshot steps
    (src/main_p3t.cpp:543-547): clusters, isolated bodies, the largest
    cluster -- and, beside it, the value GPLUM's
    getNumberOfParticleInLargestClusterLocal returns (src/hard.h:143-149): its
    test compares with the cluster count instead of the running maximum, so
    it reports the size of the last cluster of its list, the one with the
    largest id_cluster (makeList orders clusters by id_cluster,
    src/hard.h:321-438)."""
    off, mem = g.cluster_lists()
    return cluster_counts(g.n, np.diff(off), g.get("id_cluster")[mem[off[:-1]]])


def cluster_counts(n, sizes, cids):
    """cluster_stats from the bodies' count n and each cluster's size and
    id_cluster."""
    sizes = np.asarray(sizes)
    out = {"n_cluster": int(len(sizes)), "n_isolated": int(n - sizes.sum()),
           "largest_cluster": int(sizes.max()) if len(sizes) else 0, "largest_cluster_as_gplum_logs": 0}
    if len(sizes):
        out["largest_cluster_as_gplum_logs"] = int(sizes[int(np.argmax(cids))])
    return out


def run(g, disk, steps, reset_step=1024, clock=None, out_dir=None, snap_every=0, snap_tmp_every=0,
        restart=False, stats=None):
    """Start-up (or a restart from out_dir/snap_tmp.dat) and tree steps up to
    `steps`; returns the energy-error trace and the collision count.  With
    out_dir: snapNNNNNN.dat (ASCII) every snap_every steps and the binary
    restart file snap_tmp.dat every snap_tmp_every steps, as GPLUM's
    outputStep / makeSnapTmp (src/main_p3t.cpp:738-764), and each step's
    collisions appended to collisionNNNNNN.dat (src/main_p3t.cpp:390-396,
    751-758); the ASCII files are written by a host thread while the next
    steps run.  With `stats` a list, the cluster counts of every snapshot
    step (cluster_stats) are appended to it."""
    import os

    from . import _lib
    from .snapshot import Header, energy7

    P = g.params
    if restart:
        h = g.read_snapshot(os.path.join(out_dir, "snap_tmp.dat"), 1)
        istep0 = int(round(h.time / P.dt_tree))
        g.prepare()
        g.tree_soft()
        g.correct(False)  # correctForceLong: the restart keeps the hard-part state (src/main_p3t.cpp:357-359)
        e_init, edisp = h.e_init, float(h.e_now[6])
        e0 = np.array([e_init[0]])
    else:
        istep0 = 0
        e0 = startup(g, disk)
        e_init, edisp = energy7(e0), 0.0
    de, ncol = [], 0

    def header(istep, e):
        return Header(time=istep * P.dt_tree, id_next=g.id_next(), e_init=e_init, e_now=energy7(e, edisp))

    if out_dir and snap_every and not restart:
        g.write_snapshot(os.path.join(out_dir, "snap%06d.dat" % 0), 0, header(0, e0), async_write=True)
    for istep in range(istep0 + 1, steps + 1):
        at_snap = snap_every and istep % snap_every == 0
        cols, e, ed = step(g, istep, reset_step, clock=clock, stats=stats if at_snap else None)
        edisp += ed
        ncol += len(cols)
        if out_dir and snap_every and len(cols):
            # collisionNNNNNN.dat holds the collisions since snapshot NNNNNN-1
            path = os.path.join(out_dir, "collision%06d.dat" % ((istep - 1) // snap_every + 1))
            _lib.check(g.lib.p3t_collisions_write(path.encode(), 1), "p3t_collisions_write")
        de.append((e[0] - e0[0] - edisp) / e0[0])
        if out_dir and snap_every and istep % snap_every == 0:
            g.write_snapshot(os.path.join(out_dir, "snap%06d.dat" % (istep // snap_every)), 0, header(istep, e),
                             async_write=True)
        if out_dir and snap_tmp_every and istep % snap_tmp_every == 0:
            g.write_snapshot(os.path.join(out_dir, "snap_tmp.dat"), 1, header(istep, e))
    if out_dir:
        g.wait_snapshot()
    return np.array(de), ncol


WORKLOADS = {
    "disk3000": "3000-body disk, 0.95-1.05 AU, m=1e-9, rms e=2h, rms i=h, dt_tree=2^-7",
    "disk8m": "8388608 planetesimals m=1.25e-11 in 0.3-3 AU, rms e=4h, rms i=2h, theta=0.5, n_group_limit=256",
    "embryos": "1048576 planetesimals m=1e-10 in 0.5-1.5 AU (rms e=6h, rms i=3h) + 4 embryos of 3e-7 "
               "at 0.7/0.9/1.1/1.3 AU, theta=0.5, n_group_limit=256",
}


def main():
    from . import autotune, scheduler
    from .disk import P3TParams, disk_1m_embryos, disk_3000, disk_8m
    from .p3t import GpuSystem

    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--workload", default="disk3000", choices=sorted(WORKLOADS))
    ap.add_argument("--n", type=int, default=1048576, help="planetesimals of the embryo workload")
    ap.add_argument("--schedule", default="learned", choices=["learned", "size"],
                    help="hard work-queue order: the learned cost model or cluster size")
    ap.add_argument("--a-frag", type=float, default=0.0,
                    help="KOMINAMI fragmentation a_frag (0: perfect accretion)")
    ap.add_argument("--timing", action="store_true", help="synchronised per-phase wall times")
    ap.add_argument("--plain-fp64", action="store_true",
                    help="the plain FP64 form: FP64 soft kernel, one cluster per thread/warp/CTA, size order")
    ap.add_argument("--output-dir", default=None, help="directory of the snapshot files")
    ap.add_argument("--snap-every", type=int, default=0, help="snapNNNNNN.dat (ASCII) every this many steps")
    ap.add_argument("--snap-tmp-every", type=int, default=0, help="snap_tmp.dat (binary) every this many steps")
    ap.add_argument("--restart", action="store_true", help="continue from OUTPUT_DIR/snap_tmp.dat (GPLUM -r)")
    args = ap.parse_args()
    if args.workload == "disk3000":
        P, disk = P3TParams(), disk_3000()
    elif args.workload == "disk8m":
        P, disk = P3TParams(n_group_limit=256), disk_8m()
    else:
        P, disk = P3TParams(n_group_limit=256), disk_1m_embryos(args.n)
    g = GpuSystem(P, precision=1 if args.plain_fp64 else 0)
    autotune.load(g.lib)
    model = scheduler.load(lib=g.lib) if args.schedule == "learned" and not args.plain_fp64 else None
    g.lib.p3t_set_schedule(1 if model is not None else 0)
    if args.plain_fp64:
        g.lib.p3t_set_hard_mode(1)
    if args.a_frag > 0:
        g.set_fragmentation(args.a_frag)
    clock = {} if args.timing else None
    t0 = time.perf_counter()
    if args.output_dir:
        import os

        os.makedirs(args.output_dir, exist_ok=True)
    stats = []
    de, ncol = run(g, disk, args.steps, clock=clock, out_dir=args.output_dir, snap_every=args.snap_every,
                   snap_tmp_every=args.snap_tmp_every, restart=args.restart, stats=stats)
    t = time.perf_counter() - t0
    pos = g.get("pos")
    import torch

    free, total = torch.cuda.mem_get_info()
    out = {"workload": WORKLOADS[args.workload], "steps": args.steps,
           "form": "plain FP64" if args.plain_fp64 else "mixed + batched",
           "schedule": "learned cost model" if model is not None else "size",
           "device_memory_gb": (total - free) / 1e9, "ms_per_step": 1e3 * t / max(1, args.steps),
           "a_frag": args.a_frag, "max_abs_dE_over_E": float(np.abs(de).max()) if len(de) else 0.0,
           "final_dE_over_E": float(de[-1]) if len(de) else 0.0,
           "collisions": ncol, "n_initial": len(disk["mass"]), "n_final": g.n, "wall_s": t,
           # identical for every schedule: the queue order never changes the arithmetic
           "final_state_checksum": float(np.sum(pos * np.arange(1, 4))) + float(np.sum(g.get("id")))}
    if stats:
        out["clusters_at_snapshots"] = stats
    if clock is not None:
        out["phases_s"] = clock
    print(json.dumps(out))


if __name__ == "__main__":
    main()
