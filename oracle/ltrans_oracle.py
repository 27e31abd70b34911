"""CPU oracle of the length-gauge l-space transform on the tensor cores (test infrastructure only:
the tests and nothing else import it; the product computes it on the GPU, qpc_lspace_transform and
the engine's coupling step).

The reference maps the channel values c_l of every radial point between the l basis and the
eigen-basis of the coupling (cn_transform_hl, spherical/propagator/cn_1e.hpp:101-147: a dense
l x l product).  The engine uses the eigenvectors' parity (Y10 has zero diagonal, so its eigenvalues
pair as +-s with eigenvectors v and diag((-1)^l) v) and stores, per position,
    forward   slot 2k = E_k + O_k,  slot 2k+1 = conj(E_k - O_k),  slot 2 np = Z (odd n_l)
              E_k = sum_{l even} V[k][l] c_l,  O_k = sum_{l odd} V[k][l] c_l,  Z = sum_{l even} V[np][l] c_l
    backward  c_l = sum_k V[k][l] s_k (+ V[np][l] Z) for even l,  c_l = sum_k V[k][l] d_k for odd l,
              s_k, d_k in slots 2k, 2k+1
with V [np + 1][n_l] (rows k < np: eigenvectors of +s_k; row np: the zero-eigenvalue vector).

On the GPU the real and imaginary parts of each position are two rows of one product with the
block-diagonal matrix [Ve 0; 0 Vo] of half-width KB (16 for n_l <= 32, 24 for n_l <= 48), computed
in exact 8-bit digits (slices_oracle.gemm with 8 digits of 8 bits: every row of the product, both
parities together, under one power of two) and rounded once; the combinations E +- O are then FP64
additions.  This oracle forms the same rows and the same block-diagonal matrix, so its results equal
the GPU's bit for bit wherever they are normal numbers."""
import numpy as np

from . import slices_oracle as so

NS8, BITS8 = 8, 8


def half_width(n_l):
    """KB of the block-diagonal product (0: no tensor-core form)"""
    if n_l < 1:
        return 0
    return 16 if n_l <= 32 else (24 if n_l <= 48 else 0)


def _matrix(V, n_l, forward, KB):
    ne, no = (n_l + 1) // 2, n_l // 2
    Bm = np.zeros((2 * KB, 2 * KB))
    for n in range(ne):
        for k in range(ne):
            Bm[n, k] = V[n, 2 * k] if forward else V[k, 2 * n]
    for n in range(no):
        for k in range(no):
            Bm[KB + n, KB + k] = V[n, 2 * k + 1] if forward else V[k, 2 * n + 1]
    return Bm


def transform(V, c, forward):
    """the engine's transform of c [n_pos][n_l] (complex) with V [np + 1][n_l], as the tensor-core
    kernel computes it"""
    c = np.asarray(c, dtype=np.complex128)
    n_pos, n_l = c.shape
    KB = half_width(n_l)
    assert KB, n_l
    npair = n_l // 2
    rows = np.zeros((2 * n_pos, 2 * KB))
    for part, comp in enumerate((c.real, c.imag)):
        rows[part::2, 0:(n_l + 1) // 2] = comp[:, 0::2]
        rows[part::2, KB:KB + n_l // 2] = comp[:, 1::2]
    # product rows x matrix^T: output n of a row = sum_k row[k] Bm[n][k]
    P = so.gemm(rows, _matrix(np.asarray(V, dtype=np.float64), n_l, forward, KB).T, NS8, BITS8)
    re, im = P[0::2], P[1::2]
    o_re, o_im = np.zeros((n_pos, n_l)), np.zeros((n_pos, n_l))
    if forward:
        for k in range(npair):
            Er, Ei, Or, Oi = re[:, k], im[:, k], re[:, KB + k], im[:, KB + k]
            o_re[:, 2 * k], o_im[:, 2 * k] = Er + Or, Ei + Oi
            o_re[:, 2 * k + 1], o_im[:, 2 * k + 1] = Er - Or, Oi - Ei
        if n_l & 1:
            o_re[:, 2 * npair], o_im[:, 2 * npair] = re[:, npair], im[:, npair]
    else:
        ne, no = (n_l + 1) // 2, n_l // 2
        o_re[:, 0::2], o_im[:, 0::2] = re[:, :ne], im[:, :ne]
        o_re[:, 1::2], o_im[:, 1::2] = re[:, KB:KB + no], im[:, KB:KB + no]
    out = np.empty((n_pos, n_l), dtype=np.complex128)
    out.real, out.imag = o_re, o_im
    return out


def transform_fp64(V, c, forward):
    """the same map in plain FP64 (numpy), for tolerance checks"""
    c = np.asarray(c, dtype=np.complex128)
    V = np.asarray(V, dtype=np.float64)
    n_pos, n_l = c.shape
    npair = n_l // 2
    out = np.zeros_like(c)
    if forward:
        E = c[:, 0::2] @ V[:, 0::2].T
        O = c[:, 1::2] @ V[:npair, 1::2].T if npair else np.zeros((n_pos, 0))
        for k in range(npair):
            out[:, 2 * k] = E[:, k] + O[:, k]
            out[:, 2 * k + 1] = np.conj(E[:, k] - O[:, k])
        if n_l & 1:
            out[:, 2 * npair] = E[:, npair]
    else:
        out[:, 0::2] = c[:, 0::2] @ V[:(n_l + 1) // 2, 0::2]
        if npair:
            out[:, 1::2] = c[:, 1::2] @ V[:npair, 1::2]
    return out
