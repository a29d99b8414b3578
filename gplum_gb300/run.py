"""The P3T time loop on the device: GPLUM's main loop (src/main_p3t.cpp:
289-760) without its file output, on a GpuSystem whose tree, lists and every
phase of the step stay on the GPU.

    python -m gplum_gb300.run --steps 1000

integrates the 3000-body disk (0.95-1.05 AU, m = 1e-9, rms e = 2 h,
rms i = h, dt_tree = 2^-7) and prints the relative energy error
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


def step(g, istep, reset_step=1024, r_max=40.0, r_min=0.1):
    """One tree step (src/main_p3t.cpp:423-717; r_max and r_min as in
    parameter.dat, defaults src/read.h:111-112).  Returns (collision pairs,
    energy after the step, energy dissipated in this step)."""
    g.kick()
    g.cluster()
    cols, ed = g.hard(istep)
    edisp = float(ed[0])
    g.tree_soft()
    g.correct(False)
    g.kick()
    e = g.energy()
    if len(cols):
        edisp += g.merge(len(cols))
    n_rem, e_rem = g.remove(r_max, r_min)
    edisp += e_rem
    if len(cols) or n_rem or istep % reset_step == reset_step - 1:
        g.prepare()
        g.tree_soft()
        g.correct(True)
        e = g.energy()
    return cols, e, edisp


def run(g, disk, steps, reset_step=1024):
    """Start-up and `steps` tree steps; returns the energy-error trace and
    the collision count."""
    e0 = startup(g, disk)
    edisp = 0.0
    de, ncol = [], 0
    for istep in range(1, steps + 1):
        cols, e, ed = step(g, istep, reset_step)
        edisp += ed
        ncol += len(cols)
        de.append((e[0] - e0[0] - edisp) / e0[0])
    return np.array(de), ncol


def main():
    from .disk import P3TParams, disk_3000
    from .p3t import GpuSystem

    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=1000)
    args = ap.parse_args()
    P = P3TParams()
    g = GpuSystem(P)
    t0 = time.perf_counter()
    de, ncol = run(g, disk_3000(), args.steps)
    t = time.perf_counter() - t0
    print(json.dumps({"workload": "3000-body disk, 0.95-1.05 AU, m=1e-9, dt_tree=2^-7", "steps": args.steps,
                      "max_abs_dE_over_E": float(np.abs(de).max()), "final_dE_over_E": float(de[-1]),
                      "collisions": ncol, "n_final": g.n, "wall_s": t}))


if __name__ == "__main__":
    main()
