"""CPU checks of the FP64 MLP oracle used to verify the tensor-core gradients."""
import numpy as np

from oracle import mlp64


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.standard_normal(sum(r * c + r for r, c in mlp64.SHAPES)) * 0.1
    x = mlp64.LO + (mlp64.HI - mlp64.LO) * rng.random((16, 5))
    y = rng.random((16, 3))
    _, g = mlp64.loss_and_grad(p, x, y)
    eps = 1e-6
    for i in rng.integers(0, p.size, 40):
        e = np.zeros_like(p)
        e[i] = eps
        fd = (mlp64.loss_and_grad(p + e, x, y)[0] - mlp64.loss_and_grad(p - e, x, y)[0]) / (2 * eps)
        assert abs(fd - g[i]) < 1e-7 + 1e-6 * abs(g[i])


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.001953125, 3.14159265, -2.5e-3, 0.0, 1.01171875])
    r = mlp64.bf16(v)
    # 1 + 2^-8 and 1 + 3 2^-8 are ties: to the even neighbours 1 and 1 + 2^-6
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 and r[6] == 1.015625
    assert abs(r[3] - 3.140625) < 1e-12
    assert np.all(np.abs(r - v) <= np.abs(v) * 2 ** -8)
