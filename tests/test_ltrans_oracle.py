"""The oracle of the length-gauge l-space transform on the tensor cores (oracle/ltrans_oracle.py):
its 8 x 8-bit digit product against exact rational products, and the transform against the plain
FP64 map with the engine's eigenvector table; the C ABI's argument checks (CPU only)."""
from fractions import Fraction

import numpy as np
import pytest

from conftest import engine
from oracle import ltrans_oracle as lo
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


def vtable(q, n_l, m=0):
    """the engine's table: rows k < n_l/2 = eigenvectors of +s_k (largest first), then the
    zero-eigenvalue vector for odd n_l"""
    lam, P = q.y10_eigen(n_l, m)
    npair = n_l // 2
    V = np.zeros((npair + 1, n_l))
    for k in range(npair):
        V[k] = P[n_l - 1 - k]
    if n_l & 1:
        V[npair] = P[npair]
    return V


@pytest.mark.parametrize("wide", [False, True])
def test_digit_product_exact_bound(wide):
    """8 digits of 8 bits, pairs s + t <= 7: within (K + 1) 2^(ea + eb - 59) of the exact product,
    plus its one rounding (the dropped level s + t = 8 holds 7 pairs of digits below 2^8 at weight
    2^(ea + eb - 78), the digits' truncation 2^(ea + eb - 62) per term)"""
    rng = np.random.default_rng(5 + wide)
    n, K, M = 9, 48, 11
    A = rng.standard_normal((n, K))
    B = rng.standard_normal((K, M))
    if wide:
        A *= 2.0 ** rng.integers(-300, 300, (n, 1))
        B *= 2.0 ** rng.integers(-300, 300, (1, M))
        A[2] = 0.0
        A[3, ::2] *= 2.0 ** -50
    C = so.gemm(A, B, 8, 8)
    X = _exact(A, B)
    ea, _ = so.digits(A, 8, 8)
    eb, _ = so.digits(B.T, 8, 8)
    bound = (K + 1) * np.ldexp(1.0, (ea[:, None] + eb[None, :] - 59).astype(int)) + np.abs(X) * 2.0 ** -53
    assert np.all(np.abs(C - X) <= bound)


def test_integer_digits_are_exact():
    """values with few significant bits are split without truncation: the product is exact"""
    rng = np.random.default_rng(2)
    A = rng.integers(-2 ** 20, 2 ** 20, (7, 30)).astype(float)
    B = rng.integers(-2 ** 20, 2 ** 20, (30, 5)).astype(float)
    assert np.array_equal(so.gemm(A, B, 8, 8), A @ B)


@pytest.mark.parametrize("n_l", [1, 2, 3, 8, 21, 32, 33, 41, 48])
@pytest.mark.parametrize("forward", [True, False])
def test_transform_within_fp64(n_l, forward):
    q = engine()
    V = vtable(q, n_l)
    rng = np.random.default_rng(n_l * 3 + forward)
    c = rng.standard_normal((13, n_l)) + 1j * rng.standard_normal((13, n_l))
    c[4] *= 2.0 ** 200
    c[5] = 0
    c[6] *= 2.0 ** -200
    a = lo.transform(V, c, forward)
    b = lo.transform_fp64(V, c, forward)
    # elementwise: every output is a sum of at most n_l terms |V| |c| (two such for E +- O)
    mag = lo.transform_fp64(np.abs(V), np.abs(c.real) + np.abs(c.imag), True if forward else False)
    scale = np.abs(mag.real) + np.abs(mag.imag)
    if forward:
        # E + O and E - O both bounded by the sum over all l
        scale = np.maximum(scale, np.roll(scale, 1, axis=1))
    tol = 4 * (n_l + 2) * 2.0 ** -53 * (scale + np.max(np.abs(c), axis=1, keepdims=True) * np.abs(V).max())
    assert np.all(np.abs(a - b) <= tol)


def test_half_width():
    assert [lo.half_width(n) for n in (0, 1, 32, 33, 48, 49)] == [0, 16, 16, 24, 24, 0]


@pytest.mark.parametrize("n_l", [0, 49])
def test_capi_rejects_sizes(n_l):
    q = engine()
    with pytest.raises(q.QpcError) as ei:
        q.load().qpc_lspace_transform  # the symbol exists
        c = np.zeros((3, max(n_l, 1)), complex)
        V = np.zeros((max(n_l, 1) // 2 + 1, max(n_l, 1)))
        q._check(q.load().qpc_lspace_transform(3, n_l, q._ptr(V), 1, q._ptr(c), q._ptr(c.copy())))
    assert ei.value.code == 1
