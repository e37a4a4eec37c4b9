"""The MLP oracle is pinned by central finite differences of its own FP64 loss."""
import numpy as np

from oracle import mlp as M


def random_params(rng, n_in=5, H=6, n_out=3):
    return [rng.normal(0, 0.5, (H, n_in)), rng.normal(0, 0.1, H), rng.normal(0, 0.4, (H, H)), rng.normal(0, 0.1, H),
            rng.normal(0, 0.4, (n_out, H)), rng.normal(0, 0.1, n_out)]


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    P = random_params(rng)
    X = rng.normal(size=(9, 5))
    T = rng.normal(size=(9, 3))
    _, G = M.loss_grad(P, X, T, bf16_ops=False)
    h = 1e-6
    for k, p in enumerate(P):
        flat = p.ravel()
        for i in range(0, flat.size, max(1, flat.size // 7)):
            old = flat[i]
            flat[i] = old + h
            lp, _ = M.loss_grad(P, X, T, bf16_ops=False)
            flat[i] = old - h
            lm, _ = M.loss_grad(P, X, T, bf16_ops=False)
            flat[i] = old
            fd = (lp - lm) / (2 * h)
            assert abs(fd - G[k].ravel()[i]) <= 1e-7 + 1e-6 * abs(fd), (k, i, fd, G[k].ravel()[i])


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0, 1e-30])
    r = M.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # 1 + 2^-8 is a tie -> even (1.0)
    assert r[2] == 1.0078125            # rounds up
    assert abs(r[3] + 3.140625) < 1e-12
    assert r[4] == 0.0
    assert np.all(np.abs(M.bf16(np.linspace(-4, 4, 101)) - np.linspace(-4, 4, 101)) <= 2 ** -8 * 4)


def test_adam_first_step_moves_by_lr():
    rng = np.random.default_rng(1)
    P = random_params(rng)
    G = [rng.normal(size=p.shape) for p in P]
    z = [np.zeros_like(p) for p in P]
    P1, m, v = M.adam(P, G, z, z, 1, lr=1e-3)
    for p0, p1, g in zip(P, P1, G):
        np.testing.assert_allclose(p1 - p0, -1e-3 * np.sign(g), rtol=1e-4, atol=1e-9)
