"""The block cost model's device kernels (sable_mlp_infer / _loss_grad /
_train_step) against the FP64 oracle: forward outputs, loss and every
gradient entry, one Adam step, determinism, ragged batch sizes and a short
training run."""
import ctypes

import numpy as np
import pytest

from oracle import mlp_oracle as mo
from sable_gb300 import _lib
from sable_gb300.blockmodel import MLPModel, MLPTrainer

from test_mlp_oracle import norm_of, random_features

pytestmark = pytest.mark.gpu


def setup(n, seed=0):
    rng = np.random.default_rng(seed)
    f = random_features(rng, n)
    t = rng.normal(10, 2, (n, 2)).astype(np.float32)
    mean, std = norm_of(random_features(np.random.default_rng(99), 2000))
    p = mo.init_params(seed + 1).astype(np.float32)
    p[mo.NPARAMS - 2:] = 9.0
    return f, t, mean.astype(np.float32), std.astype(np.float32), p


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 5003])
def test_infer_matches_oracle(cuda, n):
    f, t, mean, std, p = setup(n)
    out = MLPModel(p, mean, std).predict(f)
    ref, _ = mo.forward(p.astype(np.float64), f, mean.astype(np.float64), std.astype(np.float64))
    assert np.all(np.abs(out - ref) <= 1e-4 * (1 + np.abs(ref))), np.abs(out - ref).max()


@pytest.mark.parametrize("n", [1, 100, 128, 2049])
def test_loss_grad_matches_oracle(cuda, n):
    import torch
    f, t, mean, std, p = setup(n, seed=n)
    tr = MLPTrainer(p, mean, std)
    loss, grad = tr.loss_grad(torch.as_tensor(f).cuda(), torch.as_tensor(t).cuda())
    L, g = mo.loss_grad(p.astype(np.float64), f, t, mean.astype(np.float64), std.astype(np.float64))
    gg = grad.cpu().numpy().astype(np.float64)
    assert abs(float(loss) - L) <= 1e-5 * abs(L)
    scale = np.abs(g).max()
    assert np.abs(gg - g).max() <= 1e-4 * scale, (np.abs(gg - g).max(), scale)
    assert np.linalg.norm(gg - g) <= 1e-5 * np.linalg.norm(g)


def test_loss_grad_is_deterministic(cuda):
    import torch
    f, t, mean, std, p = setup(3000, seed=3)
    tr = MLPTrainer(p, mean, std)
    ft, tt = torch.as_tensor(f).cuda(), torch.as_tensor(t).cuda()
    l1, g1 = tr.loss_grad(ft, tt)
    l2, g2 = tr.loss_grad(ft, tt)
    assert torch.equal(g1, g2) and torch.equal(l1, l2)


def test_train_step_matches_oracle_adam(cuda):
    import torch
    f, t, mean, std, p = setup(1500, seed=4)
    tr = MLPTrainer(p, mean, std)
    idx = np.random.default_rng(5).permutation(1500)[:700].astype(np.int32)
    ft, tt = torch.as_tensor(f).cuda(), torch.as_tensor(t).cuda()
    loss = torch.zeros(1, device="cuda")
    lr = 1e-3
    tr.step(ft, tt, torch.as_tensor(idx).cuda(), lr, loss)
    got = tr.params().astype(np.float64)
    m, s = mean.astype(np.float64), std.astype(np.float64)
    L, g = mo.loss_grad(p.astype(np.float64), f[idx], t[idx], m, s)
    want, _, _ = mo.adam_step(p.astype(np.float64), np.zeros(mo.NPARAMS), np.zeros(mo.NPARAMS), g, 1, lr)
    assert abs(float(loss) - L) <= 1e-5 * abs(L)
    big = np.abs(g) > 1e-3 * np.abs(g).max()
    assert np.abs(got - want)[big].max() <= 1e-5 * lr + 1e-6 * np.abs(want[big]).max()
    assert np.abs(got - want)[~big].max() <= 2 * lr + 1e-6


def test_training_reduces_loss(cuda):
    rng = np.random.default_rng(6)
    f = random_features(rng, 20000)
    # a smooth function of the features standing in for log2 cycles
    t = np.stack([np.log2(f[:, 0] * f[:, 1]) + 0.1 * np.log2(1 + f[:, 5]),
                  np.log2(1 + f[:, 2]) + 1.0], 1).astype(np.float32)
    mean, std = norm_of(f)
    tr = MLPTrainer(mo.init_params(7).astype(np.float32), mean.astype(np.float32), std.astype(np.float32))
    hist = tr.fit(f, t, epochs=10, batch=1024, lr=3e-3, lr_final=1e-3)
    # the same schedule run with the FP64 oracle's Adam ends near 0.03
    assert hist[-1] < 0.05 * hist[0] and hist[-1] < 0.06, hist


def test_bad_arguments_rejected(cuda):
    lib = _lib.load()
    h = ctypes.c_void_p()
    _lib.check(lib.sable_mlp_create(ctypes.byref(h)), "create")
    bad = np.array([0, 1, 1, 1, 1, 1], np.float32)
    assert lib.sable_mlp_set_norm(h, np.zeros(6, np.float32).ctypes.data, bad.ctypes.data) == -6
    assert lib.sable_mlp_loss_grad(h, None, None, 0, None, None, None) == -6
    assert lib.sable_mlp_infer(h, None, 0, None, None) == 0
    lib.sable_mlp_destroy(h)
