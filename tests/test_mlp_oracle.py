"""The FP64 block-cost-model oracle, pinned by central finite differences of
its own loss (the reference has no learned model to take vectors from)."""
import numpy as np

from oracle import mlp_oracle as mo


def random_features(rng, n):
    h = np.exp(rng.uniform(np.log(2), np.log(256), n)).astype(np.int64)
    w = np.exp(rng.uniform(np.log(2), np.log(256), n)).astype(np.int64)
    d = rng.uniform(0.01, 1.0, n)
    nnz = np.maximum(1, np.round(d * h * w))
    var = rng.uniform(0, 1, n) * (nnz / h)
    N = rng.choice([1, 8, 32, 128], n)
    return np.stack([h, w, nnz, nnz / (h * w), var, N], 1).astype(np.float32)


def norm_of(f):
    g = np.log2(1.0 + f.astype(np.float64))
    g[:, 3] = f[:, 3]
    return g.mean(0), g.std(0) + 1e-3


def test_parameter_count():
    assert mo.NPARAMS == 4738


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    f = random_features(rng, 40)
    t = rng.normal(10, 2, (40, 2))
    mean, std = norm_of(f)
    p = mo.init_params(1)
    p[mo.NPARAMS - 2:] = 9.0          # output biases near the targets
    L, g = mo.loss_grad(p, f, t, mean, std)
    assert abs(L - mo.loss(p, f, t, mean, std)) < 1e-12
    idx = rng.choice(mo.NPARAMS, 300, replace=False)
    eps = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += eps
        pm[k] -= eps
        fd = (mo.loss(pp, f, t, mean, std) - mo.loss(pm, f, t, mean, std)) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 * (1 + abs(g[k])), (k, fd, g[k])


def test_adam_first_step_is_signed_lr():
    g = np.array([1e-3, -2.0, 5.0])
    p, m1, m2 = mo.adam_step(np.zeros(3), np.zeros(3), np.zeros(3), g, 1, lr=0.01)
    np.testing.assert_allclose(p, -0.01 * np.sign(g), rtol=1e-4)


def test_transform_keeps_density():
    f = np.array([[3, 7, 5, 0.25, 0.5, 32]], np.float32)
    z = mo.transform(f, np.zeros(6), np.ones(6))
    np.testing.assert_allclose(z[0], [2, 3, np.log2(6), 0.25, np.log2(1.5), np.log2(33)], rtol=1e-7)
