"""ORACLE — test infrastructure only (tests/ and bench.py use it as the checker).

FP64 restatement of libsable's block cost model (MLP 6 -> 64 -> 64 -> 2,
ReLU): feature transform, forward pass, loss, gradient and one Adam step,
with the same parameter layout as sable_mlp_* (row-major, out x in):

    W1[64x6] b1[64] W2[64x64] b2[64] W3[2x64] b3[2]      (4738 values)

The reference has no learned cost model (it queries a pickled RandomForest,
utils/convert_real_to_vbr.py:58), so this oracle is pinned by central finite
differences of its own loss (tests/test_mlp_oracle.py), not by reference
vectors.
"""
from __future__ import annotations

import numpy as np

NF, H1, H2, NO = 6, 64, 64, 2
SHAPES = [("W1", (H1, NF)), ("b1", (H1,)), ("W2", (H2, H1)), ("b2", (H2,)), ("W3", (NO, H2)), ("b3", (NO,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    assert p.size == NPARAMS
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def pack(d) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def transform(feat, mean, std):
    """g = log2(1 + f) for every feature but density (column 3); z = (g - mean) / std."""
    f = np.asarray(feat, dtype=np.float64)
    g = np.log2(1.0 + f)
    g[:, 3] = f[:, 3]
    return (g - np.asarray(mean, np.float64)) / np.asarray(std, np.float64)


def forward(params, feat, mean, std):
    P = unpack(params)
    x = transform(feat, mean, std)
    z1 = x @ P["W1"].T + P["b1"]
    h1 = np.maximum(z1, 0)
    z2 = h1 @ P["W2"].T + P["b2"]
    h2 = np.maximum(z2, 0)
    o = h2 @ P["W3"].T + P["b3"]
    return o, (x, h1, h2)


def loss(params, feat, target, mean, std) -> float:
    o, _ = forward(params, feat, mean, std)
    n = o.shape[0]
    return float(((o - target) ** 2).sum() / (2 * n))


def loss_grad(params, feat, target, mean, std):
    """(L, dL/dparams) with L = 1/(2n) sum (o - t)^2."""
    P = unpack(params)
    o, (x, h1, h2) = forward(params, feat, mean, std)
    n = o.shape[0]
    e = o - np.asarray(target, np.float64)
    L = float((e ** 2).sum() / (2 * n))
    dO = e / n
    g = {"W3": dO.T @ h2, "b3": dO.sum(0)}
    dz2 = (dO @ P["W3"]) * (h2 > 0)
    g["W2"] = dz2.T @ h1
    g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ P["W2"]) * (h1 > 0)
    g["W1"] = dz1.T @ x
    g["b1"] = dz1.sum(0)
    return L, pack(g)


def adam_step(params, m1, m2, grad, step: int, lr: float, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update (step counts from 1); returns new (params, m1, m2)."""
    m1 = beta1 * m1 + (1 - beta1) * grad
    m2 = beta2 * m2 + (1 - beta2) * grad * grad
    mh = m1 / (1 - beta1 ** step)
    vh = m2 / (1 - beta2 ** step)
    return params - lr * mh / (np.sqrt(vh) + eps), m1, m2


def init_params(seed: int = 0) -> np.ndarray:
    """He-uniform initial weights, zero biases."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in SHAPES:
        if name.startswith("W"):
            lim = np.sqrt(6.0 / shape[1])
            d[name] = rng.uniform(-lim, lim, size=shape)
        else:
            d[name] = np.zeros(shape)
    return pack(d)
