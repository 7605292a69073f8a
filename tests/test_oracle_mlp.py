"""The FP64 oracle of the preconditioner network (oracle/mlp.py) checked on the
CPU: its analytic gradient against central finite differences of its own loss,
and its bfloat16 emulation against plain FP64 (close, not equal)."""
import numpy as np

from oracle import mlp


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.standard_normal(mlp.P_COUNT) * 0.2
    x = mlp.bf16(rng.standard_normal((60, 64)))
    t = rng.standard_normal(60)
    _, g = mlp.loss_and_grad(p, x, t, emulate=False)
    idx = rng.choice(mlp.P_COUNT, 80, replace=False)
    fd = mlp.finite_difference(p, x, t, idx, 1e-5)
    assert np.abs(fd - g[idx]).max() <= 1e-7 * max(1.0, np.abs(g[idx]).max())


def test_bf16_rounding_and_emulation():
    assert mlp.bf16(np.float32([1.0, 1.00390625, 1.005859375]))[1] == 1.0        # tie to even
    assert mlp.bf16(np.float32([1.005859375]))[0] == 1.0078125
    rng = np.random.default_rng(1)
    p = rng.standard_normal(mlp.P_COUNT) * 0.2
    x = mlp.bf16(rng.standard_normal((40, 64)))
    ye, _ = mlp.forward(p, x, True)
    y, _ = mlp.forward(p, x, False)
    assert np.abs(ye - y).max() <= 3e-2 * np.abs(y).max()
