"""Tensor-core MLP kernels against the numpy oracle (oracle/mlp.py): forward, loss, gradients
(BF16 operands, FP32 accumulation: relative L2 error per tensor <= 2e-2), Adam, training."""
import numpy as np
import pytest

from oracle import mlp as M

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


def data(n=300, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, 22)).astype(np.float32)
    T = (0.5 * np.tanh(X[:, :19] * 0.7) + 0.1 * rng.normal(size=(n, 19))).astype(np.float32)
    return X, T


def test_forward_loss_and_gradients(gpu):
    net = gpu.Mlp(22, 128, 19, seed=3)
    P = [p.astype(np.float64) for p in net.get_params()]
    X, T = data()
    Y = net.forward(X)
    Yo, _ = M.forward(P, X)
    assert rel(Y, Yo) < 1e-2
    loss = net.loss_grad(X, T)
    lo, Go = M.loss_grad(P, X, T)
    assert abs(loss - lo) / lo < 1e-2
    for g, go in zip(net.get_grads(), Go):
        assert rel(g, go) < 2e-2, (g.shape, rel(g, go))
    # the padded rows (300 is not a multiple of 64) contribute nothing: the same data tiled
    # twice gives the same mean loss and gradients
    loss2 = net.loss_grad(np.concatenate([X, X]), np.concatenate([T, T]))
    assert abs(loss2 - loss) / loss < 1e-3


def test_adam_step_matches_oracle(gpu):
    net = gpu.Mlp(22, 128, 19, seed=4)
    P = [p.astype(np.float64) for p in net.get_params()]
    X, T = data(256, 1)
    net.loss_grad(X, T)
    G = [g.astype(np.float64) for g in net.get_grads()]
    net.adam_step(lr=1e-3)
    P1 = net.get_params()
    z = [np.zeros_like(p) for p in P]
    Po, _, _ = M.adam(P, G, z, z, 1, lr=1e-3)
    for a, b in zip(P1, Po):
        np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-7)


def test_set_params_roundtrip_and_training(gpu):
    net = gpu.Mlp(22, 128, 19, seed=5)
    P = net.get_params()
    P2 = [p * 0.5 for p in P]
    net.set_params(P2)
    for a, b in zip(net.get_params(), P2):
        np.testing.assert_array_equal(a, b)
    X, T = data(4096, 2)
    l0 = net.loss_grad(X, T)
    for _ in range(300):
        net.loss_grad(X, T)
        net.adam_step(lr=3e-3)
    assert net.loss_grad(X, T) < 0.2 * l0
