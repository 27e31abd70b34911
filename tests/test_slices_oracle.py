"""The slice-product oracle (oracle/slices_oracle.py) against exact rational products: the
digits rebuild every element to 2^-63 of its row's power of two, the product stays within
(K + 1) 2^(ea + eb - 60) plus one rounding of the exact product, and within the FP64 GEMM bound of
numpy's product (CPU only)."""
from fractions import Fraction

import numpy as np

from oracle import slices_oracle as so


def _exact(A, B):
    n, K = A.shape
    M = B.shape[1]
    C = np.zeros((n, M))
    for i in range(n):
        fa = [Fraction(x) for x in A[i]]
        for j in range(M):
            C[i, j] = float(sum(fa[k] * Fraction(B[k, j]) for k in range(K)))
    return C


def _case(seed, n, K, M, wide=False):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, K))
    B = rng.standard_normal((K, M))
    if wide:
        A *= 2.0 ** rng.integers(-200, 200, (n, 1))
        B *= 2.0 ** rng.integers(-200, 200, (1, M))
        A[1] = 0.0
        B[:, 2] = 0.0
        A[3, :4] = 7e-318
    return A, B


def test_digits_rebuild_rows():
    A, _ = _case(1, 9, 37, 3, wide=True)
    e, D = so.digits(A)
    scale = 2.0 ** e[:, None]
    rebuilt = sum(D[s] * 2.0 ** (-so.BITS * (s + 1)) for s in range(so.NS)) * scale
    assert np.all(np.abs(D) <= 127)
    assert np.all(np.abs(rebuilt - A) <= 2.0 ** -63 * scale)


def test_against_exact_products():
    for seed, (n, K, M), wide in ((2, (7, 19, 5), False), (3, (6, 40, 6), True), (4, (3, 130, 4), False)):
        A, B = _case(seed, n, K, M, wide)
        C = so.gemm(A, B)
        ex = _exact(A, B)
        bound = np.abs(A) @ np.abs(B)
        ea, _ = so.digits(A)
        eb, _ = so.digits(B.T)
        scale = 2.0 ** (ea[:, None] + eb[None, :]).astype(np.float64)
        tol = (K + 1) * 2.0 ** -60 * scale + 2.0 ** -53 * np.abs(ex) + 2.0 ** -1074 * (K + 2)
        assert np.all(np.abs(C - ex) <= tol), (seed, n, K, M)
        ref = A @ B
        assert np.all(np.abs(C - ref) <= 4 * (K + 2) * 2.0 ** -53 * bound + (K + 2) * 2.0 ** -1074)
