"""CPU restatement of the learned scheduler's network and features.
TEST INFRASTRUCTURE ONLY: tests/ use it to check the device kernels of
gplum_gb300/csrc/sched.cu (forward pass, loss gradient, cluster features).

The network is a 4-32-32-1 MLP with tanh hidden units.  Parameters are one
flat vector in the device layout: W1[32][4], b1[32], W2[32][32], b2[32],
w3[32], b3.  ``norm`` = feature mean[4], feature scale[4], target mean,
target scale; inputs enter as (x - mean) * scale and predictions leave as
out / scale + mean.  Everything here is float64.
"""
import numpy as np

IN, H = 4, 32
NP = H * IN + H + H * H + H + H + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + H * IN].reshape(H, IN); o += H * IN
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def standardise(x, y, norm):
    norm = np.asarray(norm, dtype=np.float64)
    xn = (np.asarray(x, np.float64) - norm[:IN]) * norm[IN:2 * IN]
    yn = None if y is None else (np.asarray(y, np.float64) - norm[2 * IN]) * norm[2 * IN + 1]
    return xn, yn


def forward(p, xn):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    h1 = np.tanh(xn @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return h2 @ w3 + b3, h1, h2


def predict(p, norm, x):
    xn, _ = standardise(x, None, norm)
    out, _, _ = forward(p, xn)
    return out / norm[2 * IN + 1] + norm[2 * IN]


def loss_grad(p, norm, x, y):
    """0.5 mean((f(xn) - yn)^2) and its gradient in the flat layout."""
    xn, yn = standardise(x, y, norm)
    W1, b1, W2, b2, w3, b3 = unpack(p)
    out, h1, h2 = forward(p, xn)
    e = out - yn
    n = len(e)
    dz2 = (e[:, None] * w3[None, :]) * (1.0 - h2 * h2)
    dz1 = (dz2 @ W2) * (1.0 - h1 * h1)
    g = np.concatenate([(dz1.T @ xn).ravel(), dz1.sum(0), (dz2.T @ h1).ravel(), dz2.sum(0), h2.T @ e,
                        [e.sum()]]) / n
    return 0.5 * np.mean(e * e), g


def cluster_features(off, members, pos, vel, r_out_inv, dt, pairs, dt_tree):
    """Features of each cluster (rows [log2 n, log2 min sep/r_out,
    log2(1e-6 + max |dv| dt_tree / r_out), log2(dt_tree / min dt)]) from the
    cluster lists and the neighbour pairs (i, j) of the last correction."""
    nc = len(off) - 1
    cl = np.full(len(pos), -1, np.int64)
    for c in range(nc):
        cl[members[off[c]:off[c + 1]]] = c
    sep = np.full(nc, 3.0e38)
    vr = np.zeros(nc)
    for i, j in pairs:
        r = min(r_out_inv[i], r_out_inv[j])
        s = np.float32(np.sqrt(np.sum((pos[j] - pos[i]) ** 2)) * r)
        v = np.float32(np.sqrt(np.sum((vel[j] - vel[i]) ** 2)) * dt_tree * r)
        c = cl[i]
        sep[c] = min(sep[c], s)
        vr[c] = max(vr[c], v)
    dtm = np.full(nc, 3.0e38)
    for c in range(nc):
        dtm[c] = np.min(dt[members[off[c]:off[c + 1]]].astype(np.float32))
    X = np.zeros((nc, 4))
    X[:, 0] = np.log2(np.diff(off))
    X[:, 1] = np.log2(np.clip(sep, 1e-6, 1e6))
    X[:, 2] = np.log2(1e-6 + np.minimum(vr, 1e6))
    X[:, 3] = np.log2(dt_tree / np.clip(dtm, 1e-30, 1e30))
    return X
