"""CPU oracle of the slice-product FP64 GEMM (test infrastructure only: the tests and nothing else
import it; the product computes it on the GPU, qpc_dgemm_slices).

No reference code: the velocity-gauge transforms of the reference are dense FP64 products
(cn_1e.hpp:212-290, cblas/MKL); this restates the engine's way of computing them exactly.
Every row i of A (column j of B) is cut into 9 digits of 7 bits under the power of two
2^e_i of its largest element: Y = trunc(|a| 2^(63 - e_i)) as an integer below 2^63, digit s = bits
56 - 7 s .. 62 - 7 s of Y with the sign of a.  The product keeps the digit pairs with s + t <= 8:

    C_ij = 2^(e_i + f_j) sum_{s + t <= 8} 2^-7(s+t+2) sum_k alpha_s,ik beta_t,kj

summed exactly (Python integers) and rounded to FP64 once.  The GPU kernel forms the same exact sum
(fp32 tensor accumulation of integers below 2^24, int64 across chunks) and rounds it once, so its
results equal this oracle's bit for bit wherever C_ij is a normal number (a subnormal result is
rounded twice on the GPU, by the final scaling)."""
from fractions import Fraction

import numpy as np

NS, BITS = 9, 7


def _row_exponents(M):
    """frexp exponent of the largest |x| of every row: |x| < 2^e (-1022 for a row of zeros and
    subnormals)"""
    f = ((M.view(np.int64) >> 52) & 0x7FF).max(axis=1)
    return np.where(f > 0, f - 1022, -1022).astype(np.int64)


def digits(M, ns=NS, bits=BITS):
    """(e [rows], D [ns][rows][cols] int64): the signed digits of every row of M (ns digits of `bits`
    bits; 9 x 7 for the slice-product GEMM, 8 x 8 for the l-space transform)"""
    M = np.ascontiguousarray(M, dtype=np.float64)
    e = _row_exponents(M)
    b = M.view(np.int64)
    fe = (b >> 52) & 0x7FF
    m = (b & 0xFFFFFFFFFFFFF) | np.where(fe > 0, 1 << 52, 0)
    E = np.where(fe > 0, fe - 1023, -1022)
    sh = E + 11 - e[:, None]
    Y = np.zeros(M.shape, dtype=np.uint64)
    left = sh >= 0
    Y[left] = (m[left].astype(np.uint64) << sh[left].astype(np.uint64))
    right = (~left) & (sh > -64)
    Y[right] = (m[right].astype(np.uint64) >> (-sh[right]).astype(np.uint64))
    sign = np.where(b < 0, -1, 1)
    mask = np.uint64((1 << bits) - 1)
    D = np.stack([sign * ((Y >> np.uint64(bits * (ns - 1 - s))) & mask).astype(np.int64) for s in range(ns)])
    return e, D


def gemm(A, B, ns=NS, bits=BITS):
    """C = A B as the slice product defines it (digit pairs s + t < ns), correctly rounded from the
    exact digit sum"""
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    ea, da = digits(A, ns, bits)
    eb, db = digits(B.T, ns, bits)
    n, M = A.shape[0], B.shape[1]
    # exact digit-pair sums per level d = s + t (int64: each below ns K 2^(2 bits))
    lev = [sum(da[s] @ db[d - s].T for s in range(d + 1)) for d in range(ns)]
    # x = 2^(e - 63) sum_s alpha_s 2^(bits (ns - 1 - s)), so a product of two values is
    # 2^(ea + eb - 126 + bits (ns - 1)) sum_d lev_d 2^(bits (ns - 1 - d))
    C = np.zeros((n, M))
    for i in range(n):
        for j in range(M):
            tot = sum(int(lev[d][i, j]) << (bits * (ns - 1 - d)) for d in range(ns))
            e = int(ea[i] + eb[j]) - 126 + bits * (ns - 1)
            C[i, j] = float(Fraction(tot) * (Fraction(2) ** e)) if tot else 0.0
    return C
