"""The numpy network oracle is itself checked by finite differences (CPU)."""
import numpy as np

import conv_oracle as co


def test_conv_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    lattice, B = (3, 3, 2), 1
    n = sum(c_o * 27 * c_i for c_i, c_o in zip(co.CIN, co.COUT)) + sum(co.COUT)
    params = rng.standard_normal(n) * 0.2
    x = rng.standard_normal((B,) + lattice + (9,))
    y = rng.standard_normal((B,) + lattice + (3,))
    loss, grad, _ = co.loss_and_grad(params, x, y)
    idx = rng.choice(n, 40, replace=False)
    h = 1e-6
    for i in idx:
        p1 = params.copy(); p1[i] += h
        p2 = params.copy(); p2[i] -= h
        fd = (co.loss_and_grad(p1, x, y)[0] - co.loss_and_grad(p2, x, y)[0]) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-6 * max(1.0, abs(grad[i])), (i, fd, grad[i])
