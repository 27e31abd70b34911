"""CPU oracle for the surrogate MLP (qpc-tdse-cpc_gb300/csrc/qpc_mlp.cu).

TEST INFRASTRUCTURE, NOT PRODUCT CODE: only tests/ import it, as the checker.

The network has no counterpart in the reference.  This is a numpy restatement of
the engine's forward and backward pass, loss and Adam step:
  A_0 = x (zero-padded to K0 = n_in rounded up to 16)
  Z_j = A_j W_j^T + b_j,  A_{j+1} = gelu(Z_j)        (hidden layers)
  Yhat = A_{J-1} W_{J-1}^T + b_{J-1}
  loss = sum (Yhat - Y)^2 / (n n_out)
  G_{J-1} = 2 (Yhat - Y) / (n n_out)
  dW_j = G_j^T A_j,  db_j = sum_m G_j,  G_{j-1} = (G_j W_j) * gelu'(Z_{j-1})
with gelu(z) = z (1 + erf(z / sqrt 2)) / 2.  With bf16=True the values enter the
products rounded to bfloat16 where the engine rounds them (x, W, A_j for j > 0, G_j)
and the sums run in float64; with bf16=False everything is float64 (used to pin the
backward pass against finite differences).
"""
import numpy as np
from scipy.special import erf


def to_bf16(a):
    """Round float values to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = ((u + 0x7FFF + lsb) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def shapes(n_in, n_hidden, n_layers, n_out):
    K0 = (n_in + 15) // 16 * 16
    Ks = [K0] + [n_hidden] * n_layers
    Ns = [n_hidden] * n_layers + [n_out]
    return Ks, Ns


def unflatten(flat, n_in, n_hidden, n_layers, n_out):
    """The engine's flat parameter order: W_0 [N][K0], b_0, W_1, b_1, ..."""
    Ks, Ns = shapes(n_in, n_hidden, n_layers, n_out)
    out, o = [], 0
    for K, N in zip(Ks, Ns):
        W = np.asarray(flat[o:o + N * K], np.float64).reshape(N, K)
        o += N * K
        b = np.asarray(flat[o:o + N], np.float64)
        o += N
        out.append((W, b))
    return out


def flatten(params):
    return np.concatenate([np.concatenate([W.reshape(-1), b]) for W, b in params])


def loss_grad(params, X, Y, n_in, bf16=True):
    """loss and the flat gradient for rows X [n][n_in], targets Y [n][n_out]."""
    q = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    n = X.shape[0]
    K0 = params[0][0].shape[1]
    A = np.zeros((n, K0))
    A[:, :n_in] = X
    A = q(A)
    acts, zs = [A], []
    J = len(params)
    for j, (W, b) in enumerate(params):
        Z = acts[-1] @ q(W).T + b
        if j < J - 1:
            zs.append(Z)
            acts.append(q(gelu(Z)))
        else:
            Yh = Z
    n_out = Yh.shape[1]
    d = Yh - Y
    loss = float((d * d).sum() / (n * n_out))
    G = 2.0 * d / (n * n_out)
    grads = [None] * J
    for j in range(J - 1, -1, -1):
        W, b = params[j]
        Gq = q(G)
        grads[j] = (Gq.T @ acts[j], G.sum(axis=0))
        if j > 0:
            G = (Gq @ q(W)) * gelu_grad(zs[j - 1])
    g0 = grads[0][0].copy()
    g0[:, n_in:] = 0.0
    grads[0] = (g0, grads[0][1])
    return loss, flatten(grads)


def predict(params, X, n_in, bf16=True):
    q = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    K0 = params[0][0].shape[1]
    A = np.zeros((X.shape[0], K0))
    A[:, :n_in] = X
    A = q(A)
    for j, (W, b) in enumerate(params):
        Z = A @ q(W).T + b
        A = q(gelu(Z)) if j < len(params) - 1 else Z
    return A
