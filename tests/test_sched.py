"""The learned scheduler's CPU oracle: its analytic gradient against central
finite differences, and the standardisation round trip.  (The device
kernels are checked against this oracle in test_sched_gpu.py.)"""
import numpy as np

from oracle import mlp


def random_model(seed):
    rng = np.random.default_rng(seed)
    p = rng.normal(0.0, 0.3, mlp.NP)
    norm = np.concatenate([rng.normal(0, 1, 4), rng.uniform(0.5, 2.0, 4), [1.5, 0.7]])
    return p, norm


def test_oracle_gradient_matches_finite_differences():
    p, norm = random_model(1)
    rng = np.random.default_rng(2)
    x = rng.normal(0, 1.5, (200, 4))
    y = rng.normal(2, 1, 200)
    loss, g = mlp.loss_grad(p, norm, x, y)
    assert g.shape == (mlp.NP,)
    h = 1e-6
    for k in rng.choice(mlp.NP, 60, replace=False).tolist() + [0, 128, 160, 1184, 1216, 1248]:
        d = np.zeros(mlp.NP)
        d[k] = h
        num = (mlp.loss_grad(p + d, norm, x, y)[0] - mlp.loss_grad(p - d, norm, x, y)[0]) / (2 * h)
        assert abs(num - g[k]) <= 1e-6 * max(1.0, abs(g[k])), (k, num, g[k])


def test_prediction_is_destandardised():
    p, norm = random_model(3)
    x = np.random.default_rng(4).normal(0, 1, (10, 4))
    xn, _ = mlp.standardise(x, None, norm)
    out, _, _ = mlp.forward(p, xn)
    np.testing.assert_allclose(mlp.predict(p, norm, x), out / norm[9] + norm[8])
