"""Whole P3T tree steps per second on one GB300: GPLUM's main loop
(src/main_p3t.cpp:423-717) on a 1,048,576-body disk, the mixed-precision
batched form against the plain-FP64 form, in one run.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--no-extras]

Workload: the batched-hard-part disk (1,048,576 bodies, 0.95-1.05 AU,
m = 7e-11, rms e = 6 h, rms i = 3 h, theta 0.5, n_group_limit 256,
dt_tree 2^-7, perfect accretion): ~115,700 neighbour clusters of 2 to ~260
bodies per step.  One step = one p3t_tree_step call: kick, cluster labels
and lists, the hard part (every cluster in one persistent launch, learned
queue order, Kepler drift of the isolated bodies), device octree +
interaction lists + soft force, FP64 cutoff correction and neighbour search,
kick, energy, merge, out-of-boundary removal and the re-force pass after
collisions.  State resident in HBM (0.34 GB, larger than L2); each step is
timed by CUDA events on the library stream.

Printed JSON line: `value` = mixed + batched steps/s; `fp64_form` = the
plain-FP64 form (FP64 soft kernel, one cluster per thread/warp/CTA, size
order) over the same number of steps from the same initial state;
`roofline` = the hard launch (the dominant kernel) against the FP64 FMA peak
of this GPU; `accuracy` = per-body relative soft-force error against the
FP64 restatement on the step's own interaction lists, GPLUM's FP32 functor
beside it, and |dE/E| over the timed steps; `e2e` = the same steps through
the C ABI with GPLUM's FPGrav records in pinned host memory (copied in and
out every step); `cpu_baseline` = the CPU restatement of GPLUM's step (the
oracle) on the host cores.  Extras (one GPU only, skipped by --no-extras):
the soft pass alone on the 1M soft-force disk, the 1000-step embryo run with
fragmentation (learned vs size queue order) and the 8M-body large disk.

`--impl reference` times GPLUM's step arithmetic on the host cores (the CPU
restatement in oracle/, pinned bit for bit to GPLUM's own headers) on the
same disk.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_BODIES = 1048576
METRIC = "P3T steps/s, N=1M: mixed+batched vs plain FP64 on GB300 @ rel force err≤1e-6"
WORKLOAD = ("P3T tree step, 1048576-body disk 0.95-1.05 AU, m=7e-11, rms e=6h, rms i=3h, theta=0.5, "
            "n_group_limit=256, dt_tree=2^-7, perfect accretion")
# FP64 flops per evaluated hard pair term (predicted/corrected pass; full pass
# with the potential and the W cutoff), per active member and block step
# (two corrector passes, the sun force three times, the time step) and per
# member prediction (every member, every block step), FMA = 2, sqrt/div = 1
HARD_FLOPS_PC, HARD_FLOPS_FULL, HARD_FLOPS_MEMBER, HARD_FLOPS_PREDICT = 77, 120, 145, 30
EPEP_FLOPS, EPSP_FLOPS = 32, 70  # per soft pair
# DRAM bytes (read + write) per launch from the ncu captures summarised in
# profiles/ (the bench cannot read DRAM counters itself)
HARD_TRAFFIC_BYTES = 3.53e9  # 868 MB at 262,144 bodies scaled by pair terms (57.45 M / 14.15 M)
HARD_TRAFFIC_SOURCE = "ncu, profiles/k_hard_bundles_1m_hard_disk.md"
SOFT_TRAFFIC_BYTES = 195.0e6
SOFT_TRAFFIC_SOURCE = "ncu, profiles/soft_mixed_kernel_1m_disk.md"


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    def __init__(self):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", os.environ.get("LOCAL_RANK", "0")],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        if not os.path.exists(self.path):
            return None
        rows = [r.split(", ") for r in open(self.path).read().strip().splitlines() if r.strip()]
        rows = [r for r in rows if len(r) >= 9]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        reasons = set()
        for r in rows:
            for name, v in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"],
                               r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(rows[0][2]), "samples": len(rows),
                "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# the device step
def new_system(form, P):
    """A GpuSystem in one of the two forms: "mixed" (mixed soft kernel,
    bundled hard launch, learned queue order, autotuned launch shapes) or
    "plain" (FP64 soft kernel, one cluster per thread/warp/CTA, size order)."""
    from gplum_gb300 import autotune, scheduler
    from gplum_gb300.p3t import GpuSystem

    g = GpuSystem(P, precision=0 if form == "mixed" else 1)
    autotune.load(g.lib)
    g.lib.p3t_set_hard_mode(0 if form == "mixed" else 1)
    model = scheduler.load(lib=g.lib) if form == "mixed" else None
    g.lib.p3t_set_schedule(1 if model is not None else 0)
    g.lib.p3t_set_fragmentation(0.0, 10, 9.426627927538057e-12, 0)
    return g


def hard_flops(g):
    """The last hard launch: (ms, executed FP64 flops or None, algorithmic
    FP64 flops, pair terms evaluated, longest block-step chain).  Executed:
    the pair terms the launch evaluated (after its exact distance prefilter)
    plus the member phases; algorithmic: GPLUM's loop, every (active, member)
    pair three times per block step and all member pairs in the collision
    test (src/hermite.h:98-479)."""
    h = g.hard_launch_stats()
    members = HARD_FLOPS_MEMBER * h["active"] + HARD_FLOPS_PREDICT * h["predictions"]
    algorithmic = 231.0 * h["sweeps"] + 14.0 * h["coll_pairs"] + members
    executed = HARD_FLOPS_PC * h["live_pc"] + HARD_FLOPS_FULL * h["live_full"] + members
    return (h["ms"], (executed if h["counted"] else None), algorithmic, h["live_pc"] + h["live_full"],
            h["max_block_steps"])


def run_form(form, P, disk, warmup, steps, world, clocks=False, roofline=False):
    """Start-up, `warmup` untimed steps, then `steps` steps timed by the
    library's CUDA events; returns the system and a summary."""
    import torch

    g = new_system(form, P)
    g.load(disk)
    g.set_r_planet()
    e0 = g.startup()
    edisp = 0.0
    istep = 0
    for _ in range(warmup):
        istep += 1
        r = g.tree_step(istep)
        edisp += r["edisp"]
    lib = g.lib
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    _lib_sync(lib)
    launches0 = lib.p3t_launch_count()
    ms, phases, hard = [], [], []
    ncol, de_max = 0, 0.0
    t_wall = time.perf_counter()
    sampler = ClockSampler() if clocks else None
    if sampler:
        sampler.__enter__()
    try:
        for _ in range(steps):
            istep += 1
            r = g.tree_step(istep)
            ph = g.step_phases_ms()
            ms.append(sum(ph.values()))
            phases.append(ph)
            ncol += r["n_col"]
            edisp += r["edisp"]
            de_max = max(de_max, abs((r["energy"][0] - e0[0] - edisp) / e0[0]))
            if roofline:
                hard.append(hard_flops(g) + (r["n_clusters"],))
    finally:
        _lib_sync(lib)
        torch.cuda.synchronize()
        if sampler:
            sampler.__exit__()
    wall = time.perf_counter() - t_wall
    launches = lib.p3t_launch_count() - launches0
    if world > 1:
        torch.distributed.barrier()
    out = {"form": form, "steps": steps, "warmup": warmup, "ms_per_step": float(np.mean(ms)),
           "ms_per_step_min": float(np.min(ms)), "ms_per_step_max": float(np.max(ms)),
           "wall_ms_per_step": 1e3 * wall / steps,
           "phases_ms": {k: float(np.mean([p[k] for p in phases])) for k in phases[0]},
           "collisions": ncol, "n_body_end": g.n, "dE_over_E_max": de_max,
           "launches": int(launches), "istep": istep}
    if sampler:
        out["clocks"] = sampler.summary()
    if hard:
        out["hard"] = hard
    return g, out


def _lib_sync(lib):
    from gplum_gb300 import _lib
    _lib.check(lib.p3t_synchronize(), "p3t_synchronize")


def soft_accuracy(g, P):
    """Per-body relative error of the mixed soft force (the kernel's
    ForceGrav records) against the FP64 restatement of GPLUM's functors on the
    same interaction lists (the step's own device-built lists), and the same
    figures for GPLUM's FP32 functor (src/gravity_kernel.hpp:25-238)."""
    from gplum_gb300.layout import EPJ_DTYPE, FORCE_DTYPE, cleared_forces
    from gplum_gb300.soft import epi_records
    from oracle import harness as H

    g.tree_soft()
    n = g.n
    f_gpu = np.zeros(n, FORCE_DTYPE)
    from gplum_gb300 import _lib
    _lib.check(g.lib.p3t_download_forces(f_gpu.ctypes.data_as(ctypes.c_void_p), n), "p3t_download_forces")
    L = g.tree_lists(build=False)
    epj = np.zeros(n, EPJ_DTYPE)
    epj["id_local"] = np.arange(n)
    for k in ("pos", "r_out", "r_search", "id", "mass", "vel", "acc_d"):
        epj[k] = g.get(k)
    epi = epi_records(epj)
    H.CpuSystem("orc", P)  # the oracle's parameters
    lib = H.load("orc")
    vp = ctypes.c_void_p
    args = [L["n_group"]] + [L[k].ctypes.data_as(vp) for k in ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx")]
    acc4 = np.zeros(4 * n)
    ngb4 = np.zeros(4 * n, np.int32)
    dummy = cleared_forces(1)
    t0 = time.perf_counter()
    lib.orc_soft_lists(1, 0, *args, epi.ctypes.data_as(vp), epj.ctypes.data_as(vp), L["spj"].ctypes.data_as(vp),
                       dummy.ctypes.data_as(vp), acc4.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                       ngb4.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), os.cpu_count())
    t64 = time.perf_counter() - t0
    f32 = cleared_forces(n)
    lib.orc_soft_lists(0, 0, *args, epi.ctypes.data_as(vp), epj.ctypes.data_as(vp), L["spj"].ctypes.data_as(vp),
                       f32.ctypes.data_as(vp), None, None, os.cpu_count())
    a64 = acc4.reshape(n, 4)[:, :3]

    def stats(a):
        e = np.sqrt(((a.astype(np.float64) - a64) ** 2).sum(1)) / np.maximum(np.sqrt((a64 ** 2).sum(1)), 1e-300)
        return {"median": float(np.median(e)), "p99": float(np.quantile(e, 0.99)),
                "p999": float(np.quantile(e, 0.999)), "max": float(e.max()),
                "frac_le_1e-6": float((e <= 1e-6).mean())}

    same = all(np.array_equal(f_gpu[k], f32[k]) for k in ("number", "rank", "id_max", "id_min"))
    return {"bodies": n, "groups": int(L["n_group"]),
            "statistic": "per body |a - a_fp64| / |a_fp64| of the soft force, same lists",
            "mixed_kernel": stats(f_gpu["acc"]), "gplum_fp32_functor": stats(f32["acc"]),
            "neighbour_fields_equal_to_gplum_functor": bool(same), "fp64_oracle_s": t64}


def e2e_steps(g, istep0, steps):
    """Steps through the C ABI with the state in GPLUM FPGrav records in
    pinned host memory: records in, p3t_tree_step, records and collision
    records out, every step."""
    import torch

    from gplum_gb300.collisions import Record, records
    from gplum_gb300.layout import FPGRAV_DTYPE

    n = g.n
    cap = n + 65536
    host = torch.empty(cap * FPGRAV_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(FPGRAV_DTYPE)
    g.get_fpgrav(host)
    id_next = g.id_next()
    t, h2d, d2h = [], 0, 0
    istep = istep0
    for _ in range(steps):
        istep += 1
        t0 = time.perf_counter()
        m = g.n
        g.put_fpgrav(host[:m], id_next)
        r = g.tree_step(istep)
        out = g.get_fpgrav(host)
        cols = records(g.lib)
        t.append(time.perf_counter() - t0)
        id_next = g.id_next()
        h2d += m * FPGRAV_DTYPE.itemsize
        d2h += len(out) * FPGRAV_DTYPE.itemsize + len(cols) * ctypes.sizeof(Record)
        del r
    ms = float(np.mean(t)) * 1e3  # the mean, as the device-timed value
    return {"value": 1e3 / ms, "unit": "steps/s", "h2d_bytes_per_step": int(h2d // steps),
            "d2h_bytes_per_step": int(d2h // steps), "ms_per_step": ms, "steps": steps,
            "path": "p3t_state_put_fpgrav + p3t_tree_step + p3t_state_get_fpgrav + p3t_collision_records, "
                    "pinned FPGrav records"}


def hard_roofline(hard, peak64):
    """The hard launch over the timed steps: executed FP64 flops / launch
    time against the FP64 FMA peak."""
    ms = sum(h[0] for h in hard)
    ex = [h[1] for h in hard]
    alg = sum(h[2] for h in hard)
    out = {"kernel": "k_hard_bundles<256,2> (one launch per tree step)", "bound": "fp64",
           "launch_ms": ms / len(hard), "unit": "TFLOP/s", "peak": peak64,
           "peak_source": "measured (FP64 FMA microbenchmark p3t_probe_fma_peak)",
           "algorithmic_tflops": alg / (ms * 1e-3) / 1e12,
           "pair_terms_per_launch": float(np.mean([h[3] for h in hard])),
           "longest_cluster_block_steps": int(max(h[4] for h in hard)),
           "clusters_per_launch": float(np.mean([h[5] for h in hard])),
           "traffic": HARD_TRAFFIC_BYTES, "traffic_source": HARD_TRAFFIC_SOURCE,
           "flops_note": "achieved counts executed pair terms (77 flop predicted/corrected, 120 full), 145 flop "
                         "per active member and block step and 30 per member prediction; algorithmic counts "
                         "GPLUM's loop (3 n_act n pair terms and n(n-1) collision tests per block step) and the "
                         "same member work"}
    if all(x is not None for x in ex):
        out["achieved"] = sum(ex) / (ms * 1e-3) / 1e12
        out["frac"] = out["achieved"] / peak64
        out["flops_per_launch"] = sum(ex) / len(hard)
    return out


# ---------------------------------------------------------------------------
# extras
def soft_pass(P_unused=None, cpu_budget_s=5.0):
    """The soft pass alone on the 1M soft-force disk (0.5-1.5 AU, m = 1e-10):
    the fused EP-EP + EP-SP kernel over every group of the host tree's lists,
    inputs in HBM, L2 flushed between launches; its FP32 roofline and the
    functor-level e2e through p3t_soft_force_host."""
    import torch

    from gplum_gb300 import _lib, soft
    from gplum_gb300.disk import P3TParams, disk_1m_soft
    from gplum_gb300.layout import FORCE_DTYPE
    from gplum_gb300.radii import cutoff_radii
    from gplum_gb300.soft import epj_records
    from gplum_gb300.tree import build_lists

    P = P3TParams(n_group_limit=256)
    d = disk_1m_soft(N_BODIES, seed=2)
    r_out, r_search, _ = cutoff_radii(d["pos"], d["vel"], d["mass"], P)
    perm = build_lists(d["pos"], d["mass"], r_search, P.theta, P.n_leaf_limit, P.n_group_limit)["i_idx"]
    pos, vel, mass, r_out, r_search = d["pos"][perm], d["vel"][perm], d["mass"][perm], r_out[perm], r_search[perm]
    epj = epj_records(pos, vel, mass, r_out, r_search, ids=d["id"][perm])
    L = build_lists(pos, mass, r_search, P.theta, P.n_leaf_limit, P.n_group_limit)
    ni = np.diff(L["i_off"]).astype(np.int64)
    n_epep, n_epsp = int((ni * np.diff(L["j_off"])).sum()), int((ni * np.diff(L["s_off"])).sum())
    flops = EPEP_FLOPS * n_epep + EPSP_FLOPS * n_epsp
    lib = _lib.host_lib()
    from gplum_gb300 import autotune
    autotune.load(lib)
    sf = soft.SoftForce(P, precision=0)
    sf.upload_particles(epj)
    sf.upload_lists(L)
    stream = torch.cuda.ExternalStream(sf.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def timed(k, precision):
        soft.configure(P, precision=precision)
        ms = []
        for _ in range(k):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                sf.run(emit_candidates=True)
                e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return ms

    timed(3, 0)
    ms = float(np.mean(timed(10, 0)))
    ms64 = float(np.mean(timed(2, 1)))
    soft.configure(P, precision=0)
    peak = ctypes.c_double()
    _lib.check(lib.p3t_probe_fma_peak(0, ctypes.byref(peak)), "fp32 peak probe")

    def pinned(nbytes):
        return torch.empty(nbytes, dtype=torch.uint8, pin_memory=True).numpy()

    h_epj = pinned(epj.nbytes).view(epj.dtype)
    h_epj[:] = epj
    h_L = {"n_group": L["n_group"]}
    for k in ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx", "spj"):
        h_L[k] = pinned(L[k].nbytes).view(L[k].dtype)
        h_L[k][:] = L[k]
    h_force = pinned(len(epj) * FORCE_DTYPE.itemsize).view(FORCE_DTYPE)
    soft.soft_force_host(P, h_epj, h_L, out=h_force)
    e2e = []
    for _ in range(5):
        t0 = time.perf_counter()
        soft.soft_force_host(P, h_epj, h_L, out=h_force)
        e2e.append(time.perf_counter() - t0)
    achieved = flops / (ms * 1e-3) / 1e12
    out = {"workload": "soft force alone, 1048576-body disk 0.5-1.5 AU, m=1e-10, theta=0.5, n_group_limit=256, "
                       "quadrupole SPJ, tree (Morton) order, L2 flushed between launches",
           "ms_per_pass": ms, "passes_per_s": 1e3 / ms, "epep_pairs": n_epep, "epsp_pairs": n_epsp,
           "interactions_per_s": (n_epep + n_epsp) / (ms * 1e-3),
           "fp64_form_ms": ms64,
           "roofline": {"kernel": "soft_mixed_kernel", "bound": "fp32", "achieved": achieved, "peak": peak.value,
                        "unit": "TFLOP/s", "frac": achieved / peak.value,
                        "peak_source": "measured (FP32 FMA microbenchmark p3t_probe_fma_peak)",
                        "traffic": SOFT_TRAFFIC_BYTES, "traffic_source": SOFT_TRAFFIC_SOURCE},
           "e2e_passes_per_s": 1.0 / float(np.median(e2e))}
    try:
        v, sample, cores = cpu_soft_reference(L, epj, P, budget_s=cpu_budget_s)
        out["cpu_functor_port"] = {"passes_per_s": v, "cores": cores, "sample": sample}
    except Exception as e:  # the oracle is test infrastructure: report, do not fail the line
        out["cpu_functor_port"] = {"error": repr(e)}
    return out


def cpu_soft_reference(L, epj, P, budget_s=5.0):
    """GPLUM's FP32 functors (oracle restatement) on the host cores over a
    sample of the groups, scaled to the full pass by pair flops."""
    from gplum_gb300.layout import cleared_forces
    from gplum_gb300.soft import epi_records
    from oracle import harness as H

    H.CpuSystem("orc", P)
    lib = H.load("orc")
    threads = os.cpu_count()
    epi = epi_records(epj)
    ng = L["n_group"]
    vp = ctypes.c_void_p

    def run(groups):
        sub = {"n_group": len(groups)}
        for k, idx in (("i", "i_idx"), ("j", "j_idx"), ("s", "s_idx")):
            off = L[k + "_off"]
            lens = np.diff(off)[groups]
            sub[k + "_off"] = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
            sub[idx] = np.concatenate([L[idx][off[g]:off[g + 1]] for g in groups]).astype(np.int32)
        f = cleared_forces(len(epj))
        t0 = time.perf_counter()
        lib.orc_soft_lists(0, 0, sub["n_group"], *(sub[k].ctypes.data_as(vp) for k in
                                                   ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx")),
                           epi.ctypes.data_as(vp), epj.ctypes.data_as(vp), L["spj"].ctypes.data_as(vp),
                           f.ctypes.data_as(vp), None, None, threads)
        return time.perf_counter() - t0

    rng = np.random.default_rng(0)
    probe = rng.choice(ng, size=max(1, ng // 200), replace=False)
    t_probe = run(probe)
    frac = min(1.0, max(len(probe) / ng, budget_s / max(t_probe, 1e-6) * len(probe) / ng))
    groups = rng.choice(ng, size=max(1, int(frac * ng)), replace=False)
    t = run(groups)
    ni = np.diff(L["i_off"]).astype(np.int64)
    work = lambda gs: float((ni[gs] * (EPEP_FLOPS * np.diff(L["j_off"])[gs] +
                                       EPSP_FLOPS * np.diff(L["s_off"])[gs])).sum())
    step_s = t * work(np.arange(ng)) / work(groups)
    return 1.0 / step_s, f"{len(groups)} of {ng} groups ({t:.1f} s), scaled to the full pass by pair flops", threads


def long_run(workload, steps, form="mixed", schedule="learned", a_frag=0.0):
    """A run of `steps` tree steps through p3t_tree_step: wall time, hard
    launch time, collisions and the largest |dE/E| (GPLUM's calcEnergyError
    with the dissipated energy, src/energy.h:65-67)."""
    from gplum_gb300.disk import P3TParams, disk_1m_embryos, disk_8m

    P = P3TParams(n_group_limit=256)
    disk = disk_1m_embryos() if workload == "embryos" else disk_8m()
    g = new_system(form, P)
    if schedule == "size":
        g.lib.p3t_set_schedule(0)
    if a_frag > 0:
        g.set_fragmentation(a_frag)
    g.load(disk)
    g.set_r_planet()
    t0 = time.perf_counter()
    e0 = g.startup()
    edisp, de_max, ncol, hard_ms = 0.0, 0.0, 0, 0.0
    for istep in range(1, steps + 1):
        r = g.tree_step(istep)
        edisp += r["edisp"]
        ncol += r["n_col"]
        hard_ms += g.step_phases_ms()["hard"]
        de_max = max(de_max, abs((r["energy"][0] - e0[0] - edisp) / e0[0]))
    wall = time.perf_counter() - t0
    pos = g.get("pos")
    out = {"steps": steps, "form": form, "queue": schedule if form == "mixed" else "size", "a_frag": a_frag,
           "wall_s": wall, "ms_per_step": 1e3 * wall / steps, "hard_s": hard_ms * 1e-3, "collisions": ncol,
           "n_initial": len(disk["mass"]), "n_final": g.n, "max_abs_dE_over_E": de_max,
           "final_state_checksum": float(np.sum(pos * np.arange(1, 4))) + float(np.sum(g.get("id")))}
    g.lib.p3t_set_fragmentation(0.0, 10, 9.426627927538057e-12, 0)
    return out


def cpu_step_baseline(disk, P, steps):
    """GPLUM's whole tree step on the host cores: the CPU restatement (oracle)
    with the project's host tree, OpenMP over bodies and clusters as GPLUM's
    loops are; start-up not timed.  Returns (s per step, CALC_WTIME split)."""
    from oracle import harness as H

    s = H.CpuSystem("orc", P)
    lf = H.tree_lists_fn(P)
    H.p3t_init(s, disk, lf)
    clock = {}
    t0 = time.perf_counter()
    for istep in range(1, steps + 1):
        H.p3t_step(s, istep, lf, clock=clock)
    return (time.perf_counter() - t0) / steps, {k: 1e3 * v / steps for k, v in clock.items()}


def config(extra=None):
    c = {"workload": WORKLOAD, "n_bodies": N_BODIES, "theta": 0.5, "n_group_limit": 256, "n_leaf_limit": 8,
         "hard_queue": "learned cost model (gplum_gb300/sched_model.npz)", "launch_shapes": "gplum_gb300/tuning.json",
         "l2": "state larger than L2 (0.34 GB resident; soft lists and hard state re-read every step)",
         "parallelism": "replicas"}
    if extra:
        c.update(extra)
    return c


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(ms_step, world):
    """Whole-job steps/s of `world` independent replicas, each step timed as
    the slowest rank's (replicas only: no data-path collective)."""
    return world * 1e3 / ms_step


# ---------------------------------------------------------------------------
def reference_arm(args, rank, world):
    """GPLUM's whole tree step by the CPU restatement on all host cores, on
    the same disk: start-up untimed, W warm-up steps, K timed steps."""
    if rank != 0:
        return
    from gplum_gb300.disk import P3TParams, disk_1m_hard
    from oracle import harness as H

    P = P3TParams(n_group_limit=256)
    s = H.CpuSystem("orc", P)
    lf = H.tree_lists_fn(P)
    H.p3t_init(s, disk_1m_hard(N_BODIES), lf)
    istep = 0
    for _ in range(args.warmup):
        istep += 1
        H.p3t_step(s, istep, lf)
    clock, t = {}, []
    for _ in range(args.steps):
        istep += 1
        t0 = time.perf_counter()
        H.p3t_step(s, istep, lf, clock=clock)
        t.append(time.perf_counter() - t0)
    ms = 1e3 * float(np.mean(t))
    v = 1e3 / ms
    cores = os.cpu_count()
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 soft force (FP64 displacements), f64 elsewhere",
        "data": "synthetic seeded disk", "config": config(),
        "phases_ms": {k: 1e3 * x / args.steps for k, x in clock.items()},
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} whole tree steps of the same disk after {args.warmup} warm-up "
                                   "steps (start-up untimed); GPLUM's arithmetic restated in oracle/ (pinned bit "
                                   "for bit to GPLUM's headers), the project's host tree for FDPS"},
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}), flush=True)


def gpu_arm(args, rank, world):
    import torch

    from gplum_gb300 import _lib
    from gplum_gb300.disk import P3TParams, disk_1m_hard

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    P = P3TParams(n_group_limit=256)
    disk = disk_1m_hard(N_BODIES)
    warmup = max(3, args.warmup)
    g, mixed = run_form("mixed", P, disk, warmup, args.steps, world, clocks=True, roofline=True)
    lib = g.lib
    ms_step = max_over_ranks(mixed["ms_per_step"], world)
    value = replica_rate(ms_step, world)
    peak64 = ctypes.c_double()
    _lib.check(lib.p3t_probe_fma_peak(1, ctypes.byref(peak64)), "fp64 peak probe")
    roof = hard_roofline(mixed.pop("hard"), peak64.value)
    acc = soft_accuracy(g, P)
    # the same steps again, from the same start, through the C ABI with the
    # records in host memory (the device-timed run above left the state
    # `steps` steps further on, where steps take longer)
    g.load(disk)
    g.set_r_planet()
    g.startup()
    for i in range(warmup):
        g.tree_step(i + 1)
    e2e = e2e_steps(g, warmup, max(3, min(args.steps, 20)))
    del g
    _, plain = run_form("plain", P, disk, warmup, args.steps, world)
    if rank != 0:
        return
    out = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 soft force with FP64 displacements and compensated sums; f64 hard "
                                      "part, correction, drift and energy",
        "data": "synthetic seeded disk",
        "config": config({"n_collisions_timed": mixed["collisions"]}),
        "fp64_form": {"value": 1e3 / plain["ms_per_step"], "unit": "steps/s", "ms_per_step": plain["ms_per_step"],
                      "mixed_speedup": plain["ms_per_step"] / ms_step, "phases_ms": plain["phases_ms"],
                      "dE_over_E_max": plain["dE_over_E_max"], "collisions": plain["collisions"],
                      "form": "FP64 soft kernel, one cluster per thread/warp/CTA, size queue order"},
        "phases_ms": mixed["phases_ms"], "wall_ms_per_step": mixed["wall_ms_per_step"],
        "roofline": roof,
        "accuracy": {"soft_force": acc, "dE_over_E_max_timed_steps": mixed["dE_over_E_max"],
                     "dE_over_E_max_fp64_form": plain["dE_over_E_max"]},
        "e2e": e2e,
        "gpu_launches": mixed["launches"],
        "clocks": mixed.get("clocks"),
    }
    if world == 1 and not args.no_extras:
        from gplum_gb300.disk import P3TParams as PP
        try:
            cpu_s, cpu_ph = cpu_step_baseline(disk, PP(n_group_limit=256), steps=2)
            out["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                                   "sample": "2 whole tree steps of the same disk (start-up untimed), GPLUM's "
                                             "arithmetic restated in oracle/ with the project's host tree",
                                   "phases_ms": cpu_ph}
        except Exception as e:  # the oracle is test infrastructure: report, do not fail the line
            out["cpu_baseline"] = {"value": None, "unit": "steps/s", "cores": 0, "kind": "port", "sample": repr(e)}
        for key, fn in (("soft_pass", lambda: soft_pass()),
                        ("embryo_1000_learned", lambda: long_run("embryos", 1000, a_frag=0.5)),
                        ("embryo_1000_size", lambda: long_run("embryos", 1000, schedule="size", a_frag=0.5)),
                        ("disk8m_200_mixed", lambda: long_run("disk8m", 200)),
                        ("disk8m_20_plain_fp64", lambda: long_run("disk8m", 20, form="plain"))):
            if args.only_extra and key not in args.only_extra:
                continue
            try:
                out[key] = fn()
            except Exception as e:
                out[key] = {"error": repr(e)}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the CPU baseline, the soft pass alone, the embryo and the large-disk runs")
    ap.add_argument("--only-extra", nargs="*", default=None, help="run only these extras")
    ap.add_argument("--step-only", type=int, default=0, metavar="N",
                    help="start-up and one timed step of the mixed form on the N-body disk, phases printed "
                         "(a small case for profiling the step's kernels)")
    args = ap.parse_args()
    if args.step_only:
        from gplum_gb300.disk import P3TParams, disk_1m_hard
        _, r = run_form("mixed", P3TParams(n_group_limit=256), disk_1m_hard(args.step_only), 1, 1, 1)
        print(json.dumps(r))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        from oracle import harness

        harness.build_oracle(with_ref=False)
        reference_arm(args, rank, world)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    gpu_arm(args, rank, world)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
