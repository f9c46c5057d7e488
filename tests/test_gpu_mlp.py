"""The warm-start network on the tensor cores vs its CPU restatement:
forward values, gradients, and a training run that learns."""
import importlib

import numpy as np
import pytest

from oracle import mlp_ref as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def net(built_lib):
    return importlib.import_module("xpbi-webgpu_gb300.net")


def _rel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.mark.parametrize("rows", [1, 127, 128, 1000, 70000])
def test_forward_matches_reference(net, rows):
    rng = np.random.default_rng(rows)
    X = rng.standard_normal((rows, 16)).astype(np.float32)
    p = M.init(3)
    p[M.COUNT - 1] = 0.25  # nonzero output bias
    y = net.forward(X, p)
    ref, _ = M.forward(X, p)
    # bf16 re-rounding of activations can flip one ulp where f32 and f64
    # accumulation straddle a rounding boundary
    assert _rel(y, ref) < 3e-3, _rel(y, ref)


def test_gradient_matches_reference(net):
    rng = np.random.default_rng(7)
    X = rng.standard_normal((1000, 16)).astype(np.float32)
    T = rng.standard_normal(1000).astype(np.float32)
    p = M.init(5)
    g, loss = net.grad(X, T, p)
    gr, lr = M.grad(X, T, p)
    assert abs(loss - lr) <= 1e-3 * lr
    o = 0
    for name, shape in M.SIZES:
        n = int(np.prod(shape))
        e = _rel(g[o:o + n], gr[o:o + n])
        assert e < 2e-2, (name, e)
        o += n


def test_training_reduces_loss(net):
    rng = np.random.default_rng(11)
    X = rng.uniform(-1, 1, (65536, 16)).astype(np.float32)
    T = (np.sin(2 * X[:, 0]) + X[:, 1] * X[:, 2] - 0.5 * X[:, 3] ** 2).astype(np.float32)
    p0 = M.init(2)
    _, loss0 = M.grad(X[:4096], T[:4096], p0)
    p, hist = net.train(X, T, p0, steps=600, batch=4096, lr=3e-3)
    _, loss1 = M.grad(X[:4096], T[:4096], p)
    assert np.isfinite(hist).all()
    assert loss1 < 0.1 * loss0, (loss0, loss1)
