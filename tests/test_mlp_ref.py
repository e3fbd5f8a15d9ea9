"""The FP64 MLP reference (oracle/mlp_ref.py) checked by finite differences."""
import numpy as np

import mlp_ref


def test_reference_gradient_by_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, mlp_ref.P_N)
    # exactly representable weights and inputs keep bf16 rounding out of the difference quotient
    p = mlp_ref.bf16_round(p.astype(np.float32)).astype(np.float64)
    X = mlp_ref.bf16_round(rng.uniform(0, 1, (64, 16)).astype(np.float32)).astype(np.float64)
    t = rng.uniform(-1, 1, 64)
    _, g = mlp_ref.loss_and_grad(p, X, t, rnd=False)
    # the unrounded network is smooth almost everywhere: central differences
    for k in rng.choice(mlp_ref.P_N, 60, replace=False).tolist() + [mlp_ref.P_B3]:
        e = np.zeros_like(p); e[k] = 1e-6
        lp, _ = mlp_ref.loss_and_grad(p + e, X, t, rnd=False)
        lm, _ = mlp_ref.loss_and_grad(p - e, X, t, rnd=False)
        assert abs((lp - lm) / 2e-6 - g[k]) <= 1e-6 * max(1.0, abs(g[k])), k


def test_bf16_round():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-39], np.float32)
    r = mlp_ref.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.0078125) and r[3] == -2.5
