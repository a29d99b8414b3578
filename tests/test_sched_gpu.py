"""The learned scheduler on the device against its CPU oracle (oracle/mlp.py).

- forward pass and loss gradient of the device kernels vs the float64
  oracle on random models and data (FP32 kernels: 2e-4 relative);
- training on the device lowers the loss;
- the device cluster features vs the oracle's restatement from the cluster
  lists and neighbour pairs;
- ordering the hard launch by the model changes no result (bit-identical
  state and collisions), and on a held-out disk the model's order shortens
  the launch compared with size order.
"""
import ctypes
import time

import numpy as np
import pytest

from gplum_gb300 import _lib, scheduler
from gplum_gb300.disk import P3TParams, make_disk
from gplum_gb300.p3t import GpuSystem
from gplum_gb300.tree import build_lists
from oracle import mlp

pytestmark = pytest.mark.gpu
VP = ctypes.c_void_p


def random_model(seed):
    rng = np.random.default_rng(seed)
    p = rng.normal(0.0, 0.3, mlp.NP).astype(np.float32)
    norm = np.concatenate([rng.normal(0, 1, 4), rng.uniform(0.5, 2.0, 4), [1.5, 0.7]]).astype(np.float32)
    return p, norm


def test_forward_and_gradient_match_the_oracle(gpu):
    lib = _lib.host_lib()
    for seed in (1, 2):
        p, norm = random_model(seed)
        scheduler.install(p, norm, lib=lib, schedule=False)
        rng = np.random.default_rng(10 + seed)
        x = rng.normal(0, 1.5, (5000, 4)).astype(np.float32)
        y = rng.normal(2, 1, 5000).astype(np.float32)
        np.testing.assert_allclose(scheduler.predict(x, lib=lib), mlp.predict(p, norm, x), rtol=2e-4, atol=2e-4)
        loss = ctypes.c_float()
        g = np.zeros(mlp.NP, np.float32)
        _lib.check(lib.p3t_mlp_loss_grad(x.ctypes.data_as(VP), y.ctypes.data_as(VP), len(y), ctypes.byref(loss),
                                         g.ctypes.data_as(VP)), "p3t_mlp_loss_grad")
        lo, go = mlp.loss_grad(p, norm, x, y)
        assert abs(loss.value - lo) <= 2e-4 * abs(lo)
        assert np.abs(g - go).max() <= 2e-4 * np.abs(go).max(), np.abs(g - go).max() / np.abs(go).max()
    lib.p3t_mlp_reset()


def test_training_lowers_the_loss(gpu):
    lib = _lib.host_lib()
    rng = np.random.default_rng(5)
    x = rng.normal(0, 1, (40000, 4)).astype(np.float32)
    y = (np.sin(x[:, 0]) + 0.5 * x[:, 1] * x[:, 2] + 0.1 * x[:, 3]).astype(np.float32)
    hist = scheduler.train(x, y, epochs=8, batch=2048, lr=3e-3, seed=3, lib=lib)
    assert hist[-1] < 0.25 * hist[0], hist
    p, norm = scheduler.get(lib)
    pred = scheduler.predict(x, lib=lib)
    np.testing.assert_allclose(pred, mlp.predict(p, norm, x), rtol=2e-4, atol=2e-4)
    lib.p3t_mlp_reset()


def hard_disk(n, seed):
    P = P3TParams(n_group_limit=256)
    d = make_disk(n, 7e-11 * (1048576.0 / n) ** 1.5, 0.95, 1.05, ecc_hill=6.0, inc_hill=3.0, seed=seed)
    g = GpuSystem(P)
    lists = lambda: build_lists(g.get("pos"), g.get("mass"), g.get("r_search"), P.theta, P.n_leaf_limit,
                                P.n_group_limit)
    g.load(d)
    g.set_r_planet()
    g.prepare()
    for _ in range(2):
        g.soft_force(lists())
        g.correct(True)
    return g, P, lists


def test_features_match_the_oracle(gpu):
    g, P, lists = hard_disk(32768, 8)
    g.kick()
    g.cluster()
    off, mem = g.cluster_lists()
    X = g.cluster_features()
    Xo = mlp.cluster_features(off, mem, g.get("pos"), g.get("vel"), g.get("r_out_inv"), g.get("dt"), g.pairs(),
                              P.dt_tree)
    assert len(X) == len(off) - 1 > 100
    np.testing.assert_allclose(X, Xo, rtol=1e-5, atol=1e-5)


def makespan(g, istep):
    g.lib.p3t_synchronize()
    t0 = time.perf_counter()
    cols, ed = g.hard(istep)
    g.lib.p3t_synchronize()
    t = time.perf_counter() - t0
    tm = g.hard_times()
    return cols, ed, (tm[:, 1].max() - tm[:, 0].min()) * 1e-6, t * 1e3


def test_learned_order_is_exact_and_shortens_the_launch(gpu):
    lib = _lib.host_lib()
    # train on the first steps of one disk
    g, P, lists = hard_disk(131072, 9)
    log = []
    scheduler.run_steps(g, lists, 1, 4, log)
    X = np.concatenate([a for a, _ in log])
    y = scheduler.target(np.concatenate([b for _, b in log]))
    scheduler.train(X, y, epochs=40, batch=4096, lr=3e-3, seed=1, lib=lib)
    # evaluate on another disk
    g, P, lists = hard_disk(131072, 10)
    g.kick()
    g.cluster()
    assert lib.p3t_state_snapshot(0) == 0
    res = {}
    try:
        for mode in (0, 1, 0, 1):
            lib.p3t_set_schedule(mode)
            assert lib.p3t_state_snapshot(1) == 0
            cols, ed, span, wall = makespan(g, 1)
            state = [g.get(k).tobytes() for k in ("pos", "vel", "acc_d", "jerk_d", "dt", "mass", "id", "dead")]
            res.setdefault(mode, []).append((cols, ed.tobytes(), state, span, wall))
    finally:
        lib.p3t_set_schedule(0)
        lib.p3t_mlp_reset()
    a, b = res[0][0], res[1][0]
    np.testing.assert_array_equal(a[0], b[0])
    assert a[1] == b[1] and a[2] == b[2]
    span0 = min(r[3] for r in res[0])
    span1 = min(r[3] for r in res[1])
    print(f"hard launch span: size order {span0:.2f} ms, learned order {span1:.2f} ms")
    assert span1 < span0
