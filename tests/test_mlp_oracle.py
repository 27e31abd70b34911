"""The surrogate network's CPU oracle (oracle/mlp_oracle.py): bfloat16 rounding and
the backward pass against central finite differences in float64."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp_oracle as mo  # noqa: E402


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -3.14159, 0.0, 65504.0])
    r = mo.to_bf16(x)
    # 8 significant bits: 1 + 2^-8 is a tie -> even (1.0); 1 + 3 2^-8 -> 1 + 2^-6
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7 and r[3] == 1.0 + 2 ** -6
    assert abs(r[4] + 3.140625) == 0.0 and r[5] == 0.0
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    n_in, n_hidden, n_layers, n_out, n = 5, 16, 2, 8, 7
    Ks, Ns = mo.shapes(n_in, n_hidden, n_layers, n_out)
    params = [(rng.standard_normal((N, K)) * 0.5, rng.standard_normal(N) * 0.1) for K, N in zip(Ks, Ns)]
    params[0][0][:, n_in:] = 0.0
    X = rng.standard_normal((n, n_in))
    Y = rng.standard_normal((n, n_out))
    loss, g = mo.loss_grad(params, X, Y, n_in, bf16=False)
    flat = mo.flatten(params)
    idx = rng.choice(flat.size, 60, replace=False)
    K0 = Ks[0]
    for i in idx:
        if i < Ns[0] * K0 and (i % K0) >= n_in:
            continue
        h = 1e-6
        fp, fm = flat.copy(), flat.copy()
        fp[i] += h
        fm[i] -= h
        lp, _ = mo.loss_grad(mo.unflatten(fp, n_in, n_hidden, n_layers, n_out), X, Y, n_in, bf16=False)
        lm, _ = mo.loss_grad(mo.unflatten(fm, n_in, n_hidden, n_layers, n_out), X, Y, n_in, bf16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 + 1e-6 * abs(fd), (i, fd, g[i])
