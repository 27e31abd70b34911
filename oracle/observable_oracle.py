"""CPU oracle of the elliptical driver's dipole observation (test infrastructure only: the
tests and nothing else import it; the product computes it on the GPU).

observable_r (spherical/observable/1e.hpp:52-129) restated in numpy on a state
c[m][l][r] (the reference's coefficient layout, l = il + |m|):

  rm = sum over (im, il) and the partner (im + 1, il2) with l2 = l + 1 (outer) or l - 1 (inner)
       of <c_{im,il}| F |c_{im+1,il2}> * e(m, l),
       e = integrate_sinexp1 (outer) / integrate_sinexp2 (inner) (spherical/utilities/basisfunc.hpp:243-259)
  rp = sum over (im >= 1, il) and the partner (im - 1, il2) with l2 = l + 1 (inner) or l - 1 (outer)
       of <c_{im,il}| F |c_{im-1,il2}> * e'(m, l),
       e' = integrate_sinexp4 (inner) / integrate_sinexp3 (outer) (basisfunc.hpp:263-279)
  x = Re(rm + rp) / 2,  y = Im(rp - rm) / 2      (binsrc/sphTDSE.cpp:524-527)

with <a| F |b> = a^H F b for the symmetric band F[r][k] = F(r, r+k) (symb_prj_vecd)."""
import numpy as np


def band_dense(F):
    n, ne = F.shape
    A = np.zeros((n, n))
    for k in range(ne):
        idx = np.arange(n - k)
        A[idx, idx + k] = F[:n - k, k]
        A[idx + k, idx] = F[:n - k, k]
    return A


def dipole_xy(c, F, n_l, n_m, m0):
    """(x, y) of one state c [n_m][n_l][n_r] with F = <B|f(r)|B> (f = r for the dipole)."""
    c = np.asarray(c, complex).reshape(n_m, n_l, -1)
    A = band_dense(np.asarray(F, float))
    rm = 0j
    rp = 0j
    for im in range(n_m):
        m = m0 + im
        for il in range(n_l):
            l = il + abs(m)
            if im + 1 < n_m:
                m2 = m + 1
                for sgn in (+1, -1):
                    il2 = l + sgn - abs(m2)
                    if 0 <= il2 < n_l:
                        e = -np.sqrt((l + m + 2) * (l + m + 1) / ((2 * l + 1) * (2 * l + 3))) if sgn > 0 else \
                            np.sqrt((l - m) * (l - m - 1) / ((2 * l + 1) * (2 * l - 1)))
                        rm += np.vdot(c[im, il], A @ c[im + 1, il2]) * e
            if im >= 1:
                m2 = m - 1
                for sgn in (+1, -1):
                    il2 = l + sgn - abs(m2)
                    if 0 <= il2 < n_l:
                        e = np.sqrt((l - m + 2) * (l - m + 1) / ((2 * l + 1) * (2 * l + 3))) if sgn > 0 else \
                            -np.sqrt((l + m) * (l + m - 1) / ((2 * l + 1) * (2 * l - 1)))
                        rp += np.vdot(c[im, il], A @ c[im - 1, il2]) * e
    return float((rm + rp).real / 2), float((rp - rm).imag / 2)
