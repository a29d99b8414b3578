"""Learned work-queue order of the hard launch: sample collection, training
on the device, and the model file.

The hard launch takes clusters from a queue; its makespan is set by the
clusters with the longest chains of block steps.  The device model
(gplum_gb300/csrc/sched.cu) predicts log2(1 + block steps) of each cluster
from four features, and with ``p3t_set_schedule(1)`` the queue is ordered by
that prediction.  Samples are (features before the hard launch, block steps
the launch logged) of every cluster of every step of a run; training is
minibatch Adam in the device's own forward/backward kernels.

    python -m gplum_gb300.scheduler --n 1048576 --steps 9 --out gplum_gb300/sched_model.npz

collects about a million samples on the hard-part disk (1,048,576 bodies,
0.95-1.05 AU, rms e = 6 h, rms i = 3 h), trains, and writes the model.
"""
import argparse
import ctypes
import json
import os
import time

import numpy as np

from . import _lib

MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sched_model.npz")
N_PARAMS, N_NORM = 1249, 10
VP = ctypes.c_void_p


def run_steps(g, lists, istep0, steps, log=None):
    """`steps` device tree steps (src/main_p3t.cpp:423-717) of GpuSystem g;
    with `log` a list, appends (features, block steps) of each step's
    clusters.  lists: a host list builder, or None for the device tree."""

    def tree_soft():
        if lists is None:
            g.tree_soft()
        else:
            g.soft_force(lists())

    ncol = 0
    for istep in range(istep0, istep0 + steps):
        g.kick()
        g.cluster()
        X = g.cluster_features() if log is not None else None
        cols, _ = g.hard(istep)
        ncol += len(cols)
        if log is not None:
            log.append((X, g.hard_costs()[:, 0].copy()))
        tree_soft()
        g.correct(False)
        g.kick()
        if len(cols):
            g.merge(len(cols))
            g.prepare()
            tree_soft()
            g.correct(True)
    return ncol


def target(steps):
    return np.log2(1.0 + np.asarray(steps, np.float64)).astype(np.float32)


def train(X, y, epochs=30, batch=8192, lr=3e-3, seed=1, lib=None):
    """Fresh weights, then minibatch Adam on the device.  Returns the loss of
    each epoch (standardised target)."""
    lib = lib or _lib.host_lib()
    X = np.ascontiguousarray(X, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    hist = np.zeros(epochs, np.float32)
    _lib.check(lib.p3t_mlp_reset(), "p3t_mlp_reset")
    _lib.check(lib.p3t_mlp_train(X.ctypes.data_as(VP), y.ctypes.data_as(VP), len(y), epochs, batch,
                                 ctypes.c_float(lr), ctypes.c_ulonglong(seed), hist.ctypes.data_as(VP)),
               "p3t_mlp_train")
    return hist


def get(lib=None):
    lib = lib or _lib.host_lib()
    p = np.zeros(N_PARAMS, np.float32)
    nm = np.zeros(N_NORM, np.float32)
    _lib.check(lib.p3t_mlp_get(p.ctypes.data_as(VP), nm.ctypes.data_as(VP)), "p3t_mlp_get")
    return p, nm


def install(params, norm, lib=None, schedule=True):
    lib = lib or _lib.host_lib()
    p = np.ascontiguousarray(params, np.float32)
    nm = np.ascontiguousarray(norm, np.float32)
    assert p.size == N_PARAMS and nm.size == N_NORM
    _lib.check(lib.p3t_mlp_set(p.ctypes.data_as(VP), nm.ctypes.data_as(VP)), "p3t_mlp_set")
    if schedule:
        _lib.check(lib.p3t_set_schedule(1), "p3t_set_schedule")


def predict(X, lib=None):
    lib = lib or _lib.host_lib()
    X = np.ascontiguousarray(X, np.float32)
    out = np.zeros(len(X), np.float32)
    _lib.check(lib.p3t_mlp_predict(X.ctypes.data_as(VP), len(X), out.ctypes.data_as(VP)), "p3t_mlp_predict")
    return out


def save(path, params, norm, meta):
    np.savez(path, params=params, norm=norm, meta=json.dumps(meta))


def load(path=MODEL, lib=None, schedule=True):
    """Installs the model file; returns its metadata, or None when the file is
    absent (the queue then stays in size order)."""
    if not os.path.exists(path):
        return None
    z = np.load(path)
    install(z["params"], z["norm"], lib=lib, schedule=schedule)
    return json.loads(str(z["meta"]))


def main():
    from .disk import P3TParams, disk_1m_hard
    from .p3t import GpuSystem

    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1048576)
    ap.add_argument("--steps", type=int, default=9)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--out", default=MODEL)
    args = ap.parse_args()
    P = P3TParams(n_group_limit=256)
    d = disk_1m_hard(args.n)
    g = GpuSystem(P)
    g.load(d)
    g.set_r_planet()
    g.prepare()
    for _ in range(2):
        g.tree_soft()
        g.correct(True)
    log = []
    t0 = time.perf_counter()
    run_steps(g, None, 1, args.steps, log)
    X = np.concatenate([a for a, _ in log])
    y = target(np.concatenate([b for _, b in log]))
    t1 = time.perf_counter()
    hist = train(X, y, epochs=args.epochs)
    t2 = time.perf_counter()
    params, norm = get()
    pred = predict(X)
    meta = {"workload": f"hard-part disk, {args.n} bodies, 0.95-1.05 AU, rms e=6h, rms i=3h",
            "steps": args.steps, "samples": int(len(y)), "epochs": args.epochs, "loss": [float(v) for v in hist],
            "rmse_log2_steps": float(np.sqrt(np.mean((pred - y) ** 2))),
            "collect_s": t1 - t0, "train_s": t2 - t1}
    save(args.out, params, norm, meta)
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
