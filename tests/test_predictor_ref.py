"""The predictor's CPU oracle checked by finite differences (no GPU)."""
import numpy as np

from oracle import predictor_ref as R


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, R.N_PARAM)
    x = rng.uniform(0, 8, (24, R.F))
    t = rng.uniform(0, 10, 24)
    g = R.gradients(p, x, t, bf=False, dtype=np.float64)
    eps = 1e-6
    idx = list(range(0, R.N_PARAM, 97)) + [R.B1 + 3, R.B2 + 5, R.W3 + 7, R.B3]
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp = R.loss(q, x, t)
        q[i] -= 2 * eps
        lm = R.loss(q, x, t)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.0078125, -3.14159, 65504.0, 1e-30], dtype=np.float32)
    y = R.bf16(x)
    assert y[0] == 1.0 and y[1] == 1.0 and y[2] == 1.0078125  # ties to even
    assert abs(y[3] + 3.140625) < 1e-6
    assert np.all(np.abs(y - x) <= np.abs(x) * 2 ** -8)
