"""The learned-splitting network's CPU oracle (oracle/mlp_oracle.py): its
backward pass against finite differences of its forward pass (no GPU)."""
import numpy as np

import mlp_oracle as mo


def test_parameter_count_matches_abi():
    assert mo.NPARAM == 8961


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0], np.float32)
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0           # tie to even
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] + 3.140625) < 1e-7 and r[4] == 0.0


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    x = rng.normal(size=(64, 8))
    y = (rng.random(64) < 0.3).astype(float)
    norm = np.concatenate([rng.normal(size=8) * 0.1, 1.0 + rng.random(8)])
    base = mo.bf16(mo.init_params(5)).astype(np.float64)
    loss, g = mo.loss_grad(base, norm, x, y, round_bf16=False)
    loss_r, g_r = mo.loss_grad(base, norm, x, y)   # base is already BF16-exact
    assert loss == loss_r and np.array_equal(g, g_r)

    def f(p):
        return mo.loss_grad(p, norm, x, y, round_bf16=False)[0]

    for k in rng.choice(len(base), 40, replace=False):
        e = np.zeros_like(base)
        e[k] = 1e-6
        fd = (f(base + e) - f(base - e)) / 2e-6
        assert abs(fd - g[k]) < 1e-7 + 1e-5 * abs(fd), (k, fd, g[k])
