"""The CPU restatement of the warm-start network: its hand-written backward
agrees with finite differences of its own forward (bf16 rounding off)."""
import numpy as np

from oracle import mlp_ref as M


def _exact_loss(X, T, p):
    P = M.unpack(p.astype(np.float64))
    z1 = X @ P["W1"].T + P["b1"]
    a1 = M.silu(z1)
    z2 = a1 @ P["W2"].T + P["b2"]
    a2 = M.silu(z2)
    z3 = a2 @ P["W3"].T + P["b3"]
    y = M.silu(z3) @ P["w4"] + P["b4"][0]
    return ((y - T) ** 2).mean()


def test_parameter_count():
    assert M.COUNT == 9473


def test_backward_matches_finite_differences(monkeypatch):
    monkeypatch.setattr(M, "bf16", lambda x: np.asarray(x, np.float64))
    rng = np.random.default_rng(0)
    X = rng.standard_normal((40, 16))
    T = rng.standard_normal(40)
    p = M.init(1).astype(np.float64)
    g, loss = M.grad(X, T, p)
    assert abs(loss - _exact_loss(X, T, p)) < 1e-12
    idx = rng.choice(M.COUNT, 60, replace=False)
    eps = 1e-6
    for k in idx:
        pp = p.copy(); pp[k] += eps
        pm = p.copy(); pm[k] -= eps
        fd = (_exact_loss(X, T, pp) - _exact_loss(X, T, pm)) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, 3.14159265, -2.71828], np.float32)
    r = M.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: rounds to even (1.0)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] - 3.140625) < 1e-12 and abs(r[4] + 2.71875) < 1e-12
