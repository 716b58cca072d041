"""Per-(i,a)-pair MLP of the learned initial guess -- CPU oracle (test infrastructure only).

The reference has no learned component; this is the numpy statement of the network that
libcphf trains and evaluates on the GPU, used to check the GPU forward pass and gradients.

Network: u (3) -> 64 (GELU) -> 64 (GELU) -> o (2), FP32 weights packed row-major as
``W1[64,3] b1[64] W2[64,64] b2[64] W3[2,64] b3[2]``.
Inputs, from the raw features (gap ``e_a - e_i``, right-hand-side entry ``b``,
RI diagonal ``(ia|ia)``): ``u = (log gap, 10 b, 4 (ia|ia) / gap)``.
Loss per sample with targets ``(x*, d*)``:
``(b (1 + o1) - x*)^2 + (o2 - d*)^2``, averaged over the batch.
GELU is the exact form ``0.5 z (1 + erf(z / sqrt 2))``.
"""

import math

import numpy as np

H = 64
SIZES = [("W1", (H, 3)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (2, H)), ("b3", (2,))]
NWEIGHTS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(w):
    out, k = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(w[k:k + n], dtype=np.float64).reshape(shape)
        k += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SIZES])


def init_weights(seed=0):
    rng = np.random.default_rng(seed)
    d = {"W1": rng.standard_normal((H, 3)) / math.sqrt(3), "b1": np.zeros(H),
         "W2": rng.standard_normal((H, H)) / math.sqrt(H), "b2": np.zeros(H),
         "W3": rng.standard_normal((2, H)) * 0.01, "b3": np.zeros(2)}
    return pack(d).astype(np.float32)


def inputs(feat):
    """feat [n, 3] = (gap, b, (ia|ia)) -> network inputs [n, 3]."""
    feat = np.asarray(feat, dtype=np.float64)
    gap = feat[:, 0]
    return np.stack([np.log(gap), 10.0 * feat[:, 1], 4.0 * feat[:, 2] / gap], axis=1)


def _erf(z):
    return np.vectorize(math.erf)(z)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def forward(w, feat):
    p = unpack(w)
    u = inputs(feat)
    z1 = u @ p["W1"].T + p["b1"]
    h1 = gelu(z1)
    z2 = h1 @ p["W2"].T + p["b2"]
    h2 = gelu(z2)
    o = h2 @ p["W3"].T + p["b3"]
    return o, (u, z1, h1, z2, h2)


def loss_and_grad(w, feat, target):
    """Mean loss and its gradient (packed like the weights); target [n, 2] = (x*, d*)."""
    p = unpack(w)
    feat = np.asarray(feat, dtype=np.float64)
    target = np.asarray(target, dtype=np.float64)
    n = feat.shape[0]
    o, (u, z1, h1, z2, h2) = forward(w, feat)
    b = feat[:, 1]
    r1 = b * (1.0 + o[:, 0]) - target[:, 0]
    r2 = o[:, 1] - target[:, 1]
    loss = float(np.mean(r1 * r1 + r2 * r2))
    do = np.stack([2.0 * r1 * b, 2.0 * r2], axis=1) / n
    g = {"W3": do.T @ h2, "b3": do.sum(axis=0)}
    d2 = (do @ p["W3"]) * gelu_grad(z2)
    g["W2"] = d2.T @ h1
    g["b2"] = d2.sum(axis=0)
    d1 = (d2 @ p["W2"]) * gelu_grad(z1)
    g["W1"] = d1.T @ u
    g["b1"] = d1.sum(axis=0)
    return loss, pack(g)


def training_targets(b, x):
    """Targets from a converged solve: x* per element and, per (a, i) pair, the effective
    diagonal d* with x* ~ b / (1 + d*) in least squares over the right-hand sides.
    b, x: [npair, nrhs] -> (t1 [npair, nrhs], t2 [npair])."""
    num = (x * (b - x)).sum(axis=1)
    den = (x * x).sum(axis=1)
    d = np.where(den > 0, num / np.maximum(den, 1e-300), 0.0)
    return x, d
