"""The surrogate MLP's tensor-core forward and backward against the CPU
oracle (same BF16 rounding points, FP64 accumulation), and a short fit."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _data(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1, 1, (n, 8)).astype(np.float32)
    T = np.stack(
        [np.sin(2 * X[:, 0]) * X[:, 1], np.cos(X[:, 2] + X[:, 3]), X[:, 4] ** 2 + X[:, 5], X[:, 0] * X[:, 6] - X[:, 7]],
        1,
    )
    w = rng.uniform(0.5, 1.5, (n, 4)).astype(np.float32)
    return X, T.astype(np.float32), w


def test_gradients_match_oracle():
    from bldfm_gb300.mlp import MLP, param_slices
    from oracle import mlp_oracle as MO

    n = 512
    X, T, w = _data(n, 1)
    net = MLP(batch=n, seed=3)
    p = net.params()
    dev = torch.device("cuda", 0)
    Xd, Td, wd = (torch.from_numpy(a).to(dev) for a in (X, T, w))
    net.train_step(Xd, Td, wd, 0.0)
    g, loss = net.grads()
    Yo, lo, go = MO.forward_backward(p, X, T, w)
    Y = net.forward(Xd).cpu().numpy()
    assert np.linalg.norm(Y - Yo) / np.linalg.norm(Yo) < 1e-3
    assert abs(loss - lo) / lo < 1e-3
    for name, (a, b) in param_slices().items():
        ga, gb = g[a:b], go[a:b]
        err = np.linalg.norm(ga - gb) / max(np.linalg.norm(gb), 1e-30)
        assert err < 2e-3, (name, err)


def test_training_reduces_loss():
    from bldfm_gb300.mlp import MLP

    n = 4096
    X, T, w = _data(n, 2)
    dev = torch.device("cuda", 0)
    Xd, Td, wd = (torch.from_numpy(a).to(dev) for a in (X, T, w))
    net = MLP(batch=n, seed=4)
    net.train_step(Xd, Td, wd, 0.0)
    _, l0 = net.grads()
    for _ in range(300):
        net.train_step(Xd, Td, wd, 1e-3)
    net.train_step(Xd, Td, wd, 0.0)
    _, l1 = net.grads()
    assert l1 < 0.05 * l0, (l0, l1)
