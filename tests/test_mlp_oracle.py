"""The FP64 MLP oracle's gradient against central finite differences."""
import numpy as np

import mlp_oracle as M


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    params = rng.normal(0, 0.3, M.N_PARAMS)
    x = rng.normal(0, 1, (40, M.N_IN))
    t = rng.normal(0, 1, (40, M.N_OUT))
    loss, g = M.loss_and_grad(params, x, t, round_bf16=False)
    idx = rng.choice(M.N_PARAMS, 60, replace=False)
    h = 1e-6
    for i in idx:
        p1, p2 = params.copy(), params.copy()
        p1[i] += h
        p2[i] -= h
        num = (M.loss_and_grad(p1, x, t, False)[0] - M.loss_and_grad(p2, x, t, False)[0]) / (2 * h)
        assert abs(num - g[i]) <= 1e-6 + 1e-5 * abs(num), (i, num, g[i])


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159], np.float32)
    r = M.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0  # halfway rounds to even
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] - (-3.140625)) < 1e-6
