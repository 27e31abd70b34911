"""The GPU surrogate network (qpc_mlp, through the C ABI) against the numpy oracle:
forward values, loss and gradients with the same bfloat16 rounding points (sums in
fp32 on the GPU, float64 in the oracle), and training that lowers the loss."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp_oracle as mo  # noqa: E402

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n", [37, 256])
def test_loss_and_gradient_match_oracle(q, n):
    n_in, n_hidden, n_layers, n_out, E = 6, 256, 4, 384, 3
    net = q.mlp_ensemble(n_in, n_out, n_hidden, n_layers, E, seed=5)
    rng = np.random.default_rng(n)
    X = rng.standard_normal((n, n_in)).astype(np.float32)
    Y = rng.standard_normal((n, n_out)).astype(np.float32)
    loss, grad = net.loss_grad(X, Y)
    pred = net.predict(X)
    for e in range(E):
        params = mo.unflatten(net.get_params(e), n_in, n_hidden, n_layers, n_out)
        ref_loss, ref_grad = mo.loss_grad(params, X.astype(np.float64), Y.astype(np.float64), n_in)
        assert abs(loss[e] - ref_loss) <= 1e-4 * ref_loss
        assert rel(grad[e], ref_grad) < 1e-2
        # layer by layer, so that no layer hides behind a larger one
        o = 0
        for W, b in params:
            nw = W.size
            assert rel(grad[e][o:o + nw], ref_grad[o:o + nw]) < 2e-2
            o += nw + b.size
        ref_pred = mo.predict(params, X.astype(np.float64), n_in)
        assert rel(pred[e], ref_pred) < 1e-3


def test_set_get_params_round_trip(q):
    net = q.mlp_ensemble(5, 16, 32, 2, 2, seed=1)
    p = np.random.default_rng(2).standard_normal(net.n_params).astype(np.float32)
    net.set_params(1, p)
    back = net.get_params(1)
    K0 = 16
    W0 = back[:32 * K0].reshape(32, K0)
    assert np.all(W0[:, 5:] == 0)
    mask = np.ones(net.n_params, bool)
    mask[:32 * K0] = (np.arange(32 * K0) % K0) < 5
    assert np.array_equal(back[mask], p[mask])


def test_training_lowers_loss(q):
    rng = np.random.default_rng(0)
    n, n_in, n_out = 2048, 6, 64
    X = rng.uniform(-1, 1, (n, n_in)).astype(np.float32)
    w = rng.standard_normal((n_in, n_out))
    Y = np.sin(X @ w).astype(np.float32)
    net = q.mlp_ensemble(n_in, n_out, 128, 3, 5, seed=3)
    hist = net.train(X, Y, epochs=60, batch=256, lr=2e-3)
    assert np.all(hist[-1] < 0.1 * hist[0])
    pred = net.predict(X).mean(axis=0)
    assert float(np.mean((pred - Y) ** 2)) < 0.1 * float(np.mean(Y ** 2))
