"""P3T soft-force step on one GB300: GPLUM's EP-EP + EP-SP interaction pass
over a 1,048,576-body disk (0.5-1.5 AU, m = 1e-10, theta = 0.5,
n_group_limit = 256, quadrupole superparticles).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

One step = the fused EP-EP + EP-SP kernel over every i-group of the tree's
interaction lists (forces, potentials, neighbour counts and the neighbour
candidates the correction pass reads), inputs resident in HBM.  Prints one
JSON line.  `--impl reference` times GPLUM's functor arithmetic on the host
cores instead (the CPU restatement in oracle/, pinned bit-for-bit to GPLUM's
own code) on a bounded sample of the same groups.
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
METRIC = "P3T steps/s, N=1M: mixed+batched vs plain FP64 on GB300 @ rel force err\u22641e-6"
EPEP_FLOPS = 32  # per pair, FMA = 2, rsqrt/min/max/compare = 1
EPSP_FLOPS = 70
# DRAM bytes (read + write) of one pair-kernel launch on this workload, from the
# ncu capture in profiles/soft_mixed_kernel_1m_disk.md (the bench itself cannot
# read DRAM counters); refreshed with each capture
SOFT_TRAFFIC_BYTES = 195.0e6


def workload(seed=2):
    from gplum_gb300.disk import P3TParams, disk_1m_soft
    from gplum_gb300.radii import cutoff_radii
    from gplum_gb300.soft import epj_records
    from gplum_gb300.tree import build_lists

    P = P3TParams(n_group_limit=256)
    d = disk_1m_soft(N_BODIES, seed=seed)
    r_out, r_search, _ = cutoff_radii(d["pos"], d["vel"], d["mass"], P)
    # particles in the tree's (Morton) order, the order of the EPJ array FDPS
    # hands to the force kernels
    perm = build_lists(d["pos"], d["mass"], r_search, P.theta, P.n_leaf_limit, P.n_group_limit)["i_idx"]
    pos, vel, mass, r_out, r_search = d["pos"][perm], d["vel"][perm], d["mass"][perm], r_out[perm], r_search[perm]
    epj = epj_records(pos, vel, mass, r_out, r_search, ids=d["id"][perm])
    L = build_lists(pos, mass, r_search, P.theta, P.n_leaf_limit, P.n_group_limit)
    return P, epj, L


def pair_counts(L):
    ni = np.diff(L["i_off"]).astype(np.int64)
    return int((ni * np.diff(L["j_off"])).sum()), int((ni * np.diff(L["s_off"])).sum())


def config(L, extra=None):
    c = {"workload": "P3T soft force, 1048576-body disk 0.5-1.5 AU, m=1e-10, theta=0.5, "
                     "n_group_limit=256, quadrupole SPJ",
         "n_bodies": N_BODIES, "n_groups": int(L["n_group"]), "theta": 0.5, "n_group_limit": 256,
         "particle_order": "tree (Morton) order, as FDPS passes its EPJ array",
         "l2": "flushed between timed steps (256 MiB write)", "parallelism": "replicas"}
    if extra:
        c.update(extra)
    return c


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


def p3t_step_measure(precision, steps=2, n=N_BODIES, hard_mode=0, learned=True, device_tree=True):
    """The whole device P3T tree step (src/main_p3t.cpp:423-717) on the
    hard-part disk (n bodies, 0.95-1.05 AU, rms e = 6 h): kick, cluster
    labels + lists, hard part (one persistent launch), tree + interaction
    lists + soft force, correction + neighbour search, kick, energy.  Wall-clock per phase
    with the device synchronised at each phase boundary.  The octree and
    interaction lists are built on the device (tree_soft: tree + lists + soft
    force); device_tree=False builds them on the host instead.

    precision 0/1: mixed / FP64 soft force; hard_mode 0/1: bundles / one
    cluster per thread, warp or CTA; learned: queue in the order of the
    committed cost model (else size order)."""
    from gplum_gb300 import scheduler
    from gplum_gb300.disk import P3TParams, disk_1m_hard
    from gplum_gb300.p3t import GpuSystem
    from gplum_gb300.tree import build_lists

    from gplum_gb300 import autotune

    P = P3TParams(n_group_limit=256)
    d = disk_1m_hard(n)
    g = GpuSystem(P, precision=precision)
    autotune.load(g.lib)  # launch shapes chosen by gplum_gb300/autotune.py
    g.lib.p3t_set_hard_mode(hard_mode)
    model = scheduler.load(lib=g.lib) if learned else None
    g.lib.p3t_set_schedule(1 if model is not None else 0)
    ph = {}

    def lists():
        t0 = time.perf_counter()
        L = build_lists(g.get("pos"), d["mass"] if g.n == len(d["mass"]) else g.get("mass"), g.get("r_search"),
                        P.theta, P.n_leaf_limit, P.n_group_limit)
        ph["tree_host"] = ph.get("tree_host", 0.0) + time.perf_counter() - t0
        return L

    g.load(d)
    g.set_r_planet()
    g.prepare()

    def tree_soft():
        if device_tree:
            g.tree_soft()
        else:
            L = lists()
            g.soft_force(L)

    for _ in range(2):
        tree_soft()
        g.correct(True)
    e0 = g.energy()
    # warm-up of the hard path (first-use allocations, kernel loading: ~11 ms
    # once) on a copy of the state, which is then restored
    assert g.lib.p3t_state_snapshot(0) == 0
    g.kick()
    g.cluster()
    g.hard(1)
    assert g.lib.p3t_state_snapshot(1) == 0
    ph.clear()
    clusters = []
    ncol = 0

    def timed(name, fn):
        g.lib.p3t_synchronize()
        t0 = time.perf_counter()
        r = fn()
        g.lib.p3t_synchronize()
        ph[name] = ph.get(name, 0.0) + time.perf_counter() - t0
        return r

    t_all = time.perf_counter()
    for istep in range(1, steps + 1):
        timed("kick", g.kick)
        timed("cluster", g.cluster)
        cols, _ = timed("hard", lambda: g.hard(istep))
        ncol += len(cols)
        off, _m = g.cluster_lists()
        clusters.append((len(off) - 1, int(np.diff(off).max()) if len(off) > 1 else 0))
        timed("tree_soft", tree_soft)
        timed("correct", lambda: g.correct(False))
        timed("kick", g.kick)
        e = timed("energy", g.energy)
        if len(cols):
            timed("merge", lambda: g.merge(len(cols)))
            timed("radii", g.prepare)
            timed("tree_soft", tree_soft)
            timed("correct", lambda: g.correct(True))
    total = (time.perf_counter() - t_all) / steps
    g.lib.p3t_set_hard_mode(0)
    g.lib.p3t_set_schedule(0)
    ms = {k: 1e3 * v / steps for k, v in ph.items()}
    # tree_host (host list build) is nested inside tree_soft when the tree is on the host
    dev = sum(ms.values()) - 2.0 * ms.get("tree_host", 0.0)
    return {"n_bodies": n, "steps": steps, "soft": "mixed" if precision == 0 else "fp64",
            "hard": "bundles" if hard_mode == 0 else "cluster per thread/warp/CTA",
            "queue": "learned cost model" if model is not None else "size",
            "tree": "device" if device_tree else "host",
            "ms_per_step": 1e3 * total, "device_ms_per_step": dev,
            "phases_ms": ms, "clusters_per_step": [c[0] for c in clusters],
            "largest_cluster": max(c[1] for c in clusters), "collisions": ncol,
            "dE_over_E": float((e[0] - e0[0]) / e0[0])}


def cpu_step_baseline(n=N_BODIES, steps=1):
    """The same whole tree step run by GPLUM's arithmetic on the host cores
    (the oracle port, OpenMP over clusters and bodies as GPLUM's loops are),
    with the same host tree; start-up not timed.  Returns (seconds per step,
    ms per step by GPLUM's CALC_WTIME phase)."""
    from gplum_gb300.disk import P3TParams, disk_1m_hard
    from oracle import harness as H

    P = P3TParams(n_group_limit=256)
    s = H.CpuSystem("orc", P)
    lf = H.tree_lists_fn(P)
    H.p3t_init(s, disk_1m_hard(n), lf)
    clock = {}
    t0 = time.perf_counter()
    for istep in range(1, steps + 1):
        H.p3t_step(s, istep, lf, clock=clock)
    return (time.perf_counter() - t0) / steps, {k: 1e3 * v / steps for k, v in clock.items()}


def cpu_reference(L, epj, P, budget_s=20.0, threads=None):
    """GPLUM's functor arithmetic (oracle restatement, FP32 functors) on the
    host cores over a sample of the groups; returns (steps/s, sample text, cores)."""
    import ctypes

    from gplum_gb300.layout import cleared_forces
    from gplum_gb300.soft import epi_records
    from oracle import harness as H

    harness_sys = H.CpuSystem("orc", P)  # sets the oracle's parameters
    lib = harness_sys.lib
    threads = threads or os.cpu_count()
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
    work = lambda gs: float((ni[gs] * (EPEP_FLOPS * np.diff(L["j_off"])[gs] + EPSP_FLOPS * np.diff(L["s_off"])[gs])).sum())
    step_s = t * work(np.arange(ng)) / work(groups)
    return 1.0 / step_s, f"{len(groups)} of {ng} groups ({t:.1f} s), scaled to the full step by pair flops", threads


def max_over_ranks(x, world):
    """The largest x over the ranks (every rank receives it); x itself on one
    rank.  NCCL tensors live on the rank's GPU, gloo tensors on the host."""
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


def reference_arm(args, rank, world):
    if rank != 0:
        return
    P, epj, L = workload()
    steps_s = []
    for _ in range(args.warmup):
        cpu_reference(L, epj, P, budget_s=2.0)
    for _ in range(args.steps):
        v, sample, cores = cpu_reference(L, epj, P, budget_s=max(2.0, 60.0 / max(args.steps, 1)))
        steps_s.append(v)
    v = float(np.mean(steps_s))
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 displacements)",
        "data": "synthetic seeded disk", "config": config(L),
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}), flush=True)


def gpu_arm(args, rank, world):
    import torch

    from gplum_gb300 import _lib, soft
    from gplum_gb300.layout import EPJ_DTYPE, FORCE_DTYPE

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    P, epj, L = workload()
    n_epep, n_epsp = pair_counts(L)
    flops = EPEP_FLOPS * n_epep + EPSP_FLOPS * n_epsp
    lib = _lib.host_lib()

    from gplum_gb300 import autotune

    tuning = autotune.load(lib)  # work split chosen by gplum_gb300/autotune.py on this workload
    sf = soft.SoftForce(P, precision=0)
    sf.upload_particles(epj)
    sf.upload_lists(L)
    stream = torch.cuda.ExternalStream(sf.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def timed_steps(k, precision):
        soft.configure(P, precision=precision)
        ms = []
        for _ in range(k):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                sf.run(emit_candidates=True)
                e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return ms

    for _ in range(max(3, args.warmup)):
        sf.run(emit_candidates=True)
    sf.synchronize()
    _lib.check(lib.p3t_status(), "warm-up")
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler() as clk:
        ms = timed_steps(args.steps, 0)
        torch.cuda.synchronize()
    clocks = clk.summary()
    st = lib.p3t_status()
    if st not in (0,):
        raise RuntimeError(f"soft kernel reported status {st}")
    ms_step = float(np.mean(ms))
    ms_step = max_over_ranks(ms_step, world)
    value = replica_rate(ms_step, world)

    # plain FP64 form of the same kernel (the accuracy / speed baseline)
    ms64 = float(np.mean(timed_steps(2, 1)))
    soft.configure(P, precision=0)

    # FP32 pipe peak of this GPU (project microbenchmark)
    peak, peak64 = ctypes.c_double(), ctypes.c_double()
    _lib.check(lib.p3t_probe_fma_peak(0, ctypes.byref(peak)), "fp32 peak probe")
    _lib.check(lib.p3t_probe_fma_peak(1, ctypes.byref(peak64)), "fp64 peak probe")
    achieved = flops / (ms_step * 1e-3) / 1e12
    achieved64 = flops / (ms64 * 1e-3) / 1e12

    # end to end through the C ABI with pinned host buffers
    def pinned(nbytes):
        return torch.empty(nbytes, dtype=torch.uint8, pin_memory=True).numpy()

    h_epj = pinned(epj.nbytes).view(EPJ_DTYPE)
    h_epj[:] = epj
    h_L = {"n_group": L["n_group"]}
    for k in ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx", "spj"):
        h_L[k] = pinned(L[k].nbytes).view(L[k].dtype)
        h_L[k][:] = L[k]
    h_force = pinned(len(epj) * FORCE_DTYPE.itemsize).view(FORCE_DTYPE)
    soft.soft_force_host(P, h_epj, h_L, out=h_force)
    e2e = []
    for _ in range(max(2, min(args.steps, 5))):
        t0 = time.perf_counter()
        soft.soft_force_host(P, h_epj, h_L, out=h_force)
        e2e.append(time.perf_counter() - t0)
    h2d = epj.nbytes + sum(L[k].nbytes for k in ("i_off", "i_idx", "j_off", "j_idx", "s_off", "s_idx", "spj"))
    d2h = h_force.nbytes

    if rank != 0:
        return
    out = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 displacements, compensated sums)",
        "data": "synthetic seeded disk", "config": config(L, {"epep_pairs": n_epep, "epsp_pairs": n_epsp}),
        "fp64_form": {"ms_per_step": ms64, "steps_per_s": 1e3 / ms64, "mixed_speedup": ms64 / ms_step,
                      "achieved_tflops": achieved64, "fp64_peak_tflops": peak64.value},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                     "frac": achieved / peak.value, "peak_source": "measured (FP32 FMA microbenchmark)",
                     "flops_per_step": flops,
                     # DRAM bytes read + written by one launch of the pair kernel, from the
                     # ncu capture summarised in profiles/soft_mixed_kernel_1m_disk.md
                     "traffic": SOFT_TRAFFIC_BYTES, "traffic_source": "ncu, profiles/soft_mixed_kernel_1m_disk.md"},
        "interactions_per_s": (n_epep + n_epsp) / (ms_step * 1e-3),
        "e2e": {"value": 1.0 / float(np.median(e2e)), "unit": "steps/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        # per step: position splits, superparticle pack, pair kernel
        "gpu_launches": 3 * args.steps,
        "soft_tiles": tuning["soft_tiles"] if tuning else [128, 64, 32],
        "soft_ctas_per_sm": tuning.get("soft_occ", 5) if tuning else 5,
        "clocks": clocks,
    }
    if not args.skip_step:
        try:
            mixed = p3t_step_measure(0)
            plain = p3t_step_measure(1, steps=1, hard_mode=1, learned=False)
            out["p3t_step"] = {"workload": "hard-part disk, 1048576 bodies, 0.95-1.05 AU, m=7e-11, "
                                           "rms e=6h, rms i=3h, theta=0.5, n_group_limit=256",
                               "mixed_batched": mixed, "plain_fp64": plain,
                               "device_speedup": plain["device_ms_per_step"] / mixed["device_ms_per_step"],
                               "hard_speedup": plain["phases_ms"]["hard"] / mixed["phases_ms"]["hard"]}
            cpu_s, cpu_phases = cpu_step_baseline()
            out["p3t_step"]["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": "steps/s", "cores": os.cpu_count(),
                                               "kind": "port", "sample": "1 tree step, same disk and host tree",
                                               "phases_ms": cpu_phases}
        except Exception as e:
            out["p3t_step"] = {"error": repr(e)}
    try:
        v, sample, cores = cpu_reference(L, epj, P, budget_s=15.0)
        out["cpu_baseline"] = {"value": v, "unit": "steps/s", "cores": cores, "kind": "port", "sample": sample}
    except Exception as e:  # the oracle is test infrastructure; report, do not fail the GPU line
        out["cpu_baseline"] = {"value": None, "unit": "steps/s", "cores": 0, "kind": "port", "sample": str(e)}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--skip-step", action="store_true", help="skip the whole-step measurement")
    ap.add_argument("--step-only", type=int, default=0, metavar="N",
                    help="only run one whole device step on the N-body hard-part disk and print its phases "
                         "(a small case for profiling the step's kernels)")
    ap.add_argument("--hard-mode", type=int, default=0, choices=[0, 1],
                    help="with --step-only: 0 bundled hard launch (default), 1 one cluster per thread/warp/CTA")
    args = ap.parse_args()
    if args.step_only:
        print(json.dumps(p3t_step_measure(0, steps=1, n=args.step_only, hard_mode=args.hard_mode,
                                          learned=args.hard_mode == 0)))
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
