"""The FP64 product of the velocity-gauge transforms on the bf16 tensor cores (qpc_dgemm_slices,
exact digit slices, the Ozaki scheme) against an FP64 product, through the C ABI: ragged and
one-element shapes, K past the exact-chunk length (1024), rows and columns spanning hundreds of
binary orders of magnitude, zero rows and columns, subnormals.  The bound is elementwise: the
slices' truncation (2^-55) plus the FP64 reference's own rounding, times sum_k |a_ik| |b_kj|, plus
K subnormal spacings (2^-1074) for results below the normal range, where the reference's
partial sums round on that spacing (the slice product is rounded once, from the exact sum)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["mma.sync", "tcgen05", "tcgen05+tma", "tcgen05+tma, warp-specialised"], autouse=True)
def product_path(request, monkeypatch):
    """every case on each tensor-core path of the product (warp-level mma.sync; tcgen05 with the
    accumulator in tensor memory, operands by cp.async, by TMA from one thread, or by TMA with producer,
    MMA and epilogue warps), selected per call by QPC_OZ_TC and QPC_OZ_TMA"""
    monkeypatch.setenv("QPC_OZ_TC", "0" if request.param == "mma.sync" else "1")
    monkeypatch.setenv("QPC_OZ_TMA", {"tcgen05+tma": "1", "tcgen05+tma, warp-specialised": "2"}.get(request.param, "0"))
    return request.param


def _check(q, A, B, c=4.0):
    C = q.dgemm_slices(A, B)
    ref = A @ B
    bound = np.abs(A) @ np.abs(B)
    K = A.shape[1]
    tol = c * (K + 2) * 2.0 ** -53 * bound + (K + 2) * 2.0 ** -1074
    err = np.abs(C - ref)
    assert np.all(err <= tol), (float((err / np.where(bound > 0, bound, 1)).max()), K)
    return C


@pytest.mark.parametrize("n,K,M", [(1, 1, 1), (1, 17, 3), (37, 53, 29), (64, 64, 64), (65, 130, 66), (100, 1024, 70),
                                   (70, 1025, 50), (33, 2500, 41), (128, 4100, 16)])
def test_shapes(q, n, K, M):
    rng = np.random.default_rng(n * 10007 + K * 31 + M)
    A = rng.standard_normal((n, K))
    B = rng.standard_normal((K, M))
    _check(q, A, B)


def test_orthogonal_times_state_like(q):
    """the use: an orthogonal transform times vectors whose channels decay over many decades"""
    rng = np.random.default_rng(3)
    K = 300
    Q, _ = np.linalg.qr(rng.standard_normal((K, K)))
    B = rng.standard_normal((K, 200)) * np.exp(-rng.uniform(0, 60, (K, 1)))
    C = _check(q, Q, B)
    assert np.linalg.norm(C - Q @ B) <= 4e-16 * np.linalg.norm(Q @ B) * np.sqrt(K)


def test_wide_exponents_zeros_subnormals(q):
    rng = np.random.default_rng(4)
    n, K, M = 40, 90, 30
    A = rng.standard_normal((n, K)) * 2.0 ** rng.integers(-300, 300, (n, 1))
    B = rng.standard_normal((K, M)) * 2.0 ** rng.integers(-300, 300, (1, M))
    A[5] = 0.0
    B[:, 7] = 0.0
    A[9, :10] = 5e-320          # subnormal entries in an otherwise normal row
    A[11] = 3e-310              # a row of subnormals
    B[:, 3] *= 2.0 ** -20       # a column 20 binades below the others
    B[2, 4] = -1e-300
    C = _check(q, A, B)
    assert np.all(C[5] == 0.0) and np.all(C[:, 7] == 0.0)


def test_deterministic(q):
    rng = np.random.default_rng(5)
    A, B = rng.standard_normal((50, 700)), rng.standard_normal((700, 60))
    assert np.array_equal(q.dgemm_slices(A, B), q.dgemm_slices(A, B))


def test_paths_agree(q, monkeypatch):
    """both tensor-core paths form the same exact sums: identical results, tiles of either path ragged"""
    rng = np.random.default_rng(7)
    A, B = rng.standard_normal((300, 1500)), rng.standard_normal((1500, 170))
    monkeypatch.setenv("QPC_OZ_TC", "0")
    C0 = q.dgemm_slices(A, B)
    monkeypatch.setenv("QPC_OZ_TC", "1")
    monkeypatch.setenv("QPC_OZ_TMA", "0")
    assert np.array_equal(C0, q.dgemm_slices(A, B))
    monkeypatch.setenv("QPC_OZ_TMA", "1")
    assert np.array_equal(C0, q.dgemm_slices(A, B))
    monkeypatch.setenv("QPC_OZ_TMA", "2")
    assert np.array_equal(C0, q.dgemm_slices(A, B))


def test_bit_exact_against_oracle(q):
    """the kernel rounds the exact digit sum once, as the oracle does: equal bit for bit
    (normal results), including K past one exact chunk"""
    from oracle import slices_oracle as so
    rng = np.random.default_rng(6)
    for n, K, M, wide in ((9, 40, 7, False), (5, 1100, 4, False), (8, 60, 6, True)):
        A = rng.standard_normal((n, K))
        B = rng.standard_normal((K, M))
        if wide:
            A *= 2.0 ** rng.integers(-100, 100, (n, 1))
            B *= 2.0 ** rng.integers(-100, 100, (1, M))
        C = q.dgemm_slices(A, B)
        ref = so.gemm(A, B)
        normal = np.abs(ref) >= 2.0 ** -1022
        assert np.array_equal(C[normal], ref[normal]), (n, K, M)
