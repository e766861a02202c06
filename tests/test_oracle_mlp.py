"""The surrogate network's CPU restatement (oracle/mlp.py) pinned on its own:
its hand-written parameter gradient against central differences of its loss
(float64, no rounding), its input tangents against central differences of
the forward pass, and its bfloat16 rounding against torch's conversion."""
import numpy as np
import torch

from oracle import mlp


def _data(n=9, nin=4, seed=3):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (n, nin))
    y = np.sin(x).sum(axis=1)
    dy = np.cos(x)
    return x, y, dy


def test_tangents_are_the_input_gradient():
    x, _, _ = _data()
    p = mlp.init_params(4, seed=1)
    f, g, _ = mlp.forward(p, x)
    h = 1e-6
    for d in range(4):
        e = np.zeros(4)
        e[d] = h
        fp, _, _ = mlp.forward(p, x + e, tangents=False)
        fm, _, _ = mlp.forward(p, x - e, tangents=False)
        np.testing.assert_allclose(g[:, d], (fp - fm) / (2 * h), rtol=1e-6, atol=1e-8)


def test_parameter_gradient_matches_central_differences():
    x, y, dy = _data()
    p = mlp.init_params(4, seed=2)
    lam = 0.7
    loss, grad = mlp.loss_grad(p, x, y, dy, lam)
    rng = np.random.default_rng(5)
    o, _ = mlp.offsets(4)
    # a few entries of every block
    idx = []
    for name, (a, s) in o.items():
        idx += list(a + rng.choice(s, size=min(s, 6), replace=False))
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        lp, _ = mlp.loss_grad(p + e, x, y, dy, lam)
        lm, _ = mlp.loss_grad(p - e, x, y, dy, lam)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - grad[i]) < 1e-6 * max(1.0, abs(fd)), (i, fd, grad[i])


def test_bf16_rounding_matches_torch():
    v = np.random.default_rng(0).normal(size=4096) * np.exp(np.random.default_rng(1).uniform(-20, 20, 4096))
    v = np.concatenate([v, [0.0, -0.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -9]])
    ref = torch.from_numpy(v.astype(np.float32)).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(mlp.bf16_round(v), ref)
