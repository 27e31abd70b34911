"""Wavefunction files with the reference driver's dataset names and layout.

The reference writes its state to HDF5 (util::save_basic and the /coef1 dataset,
binsrc/sphTDSE.cpp:167-200, 254-259) and reads an initial state back with grid checks
(init::load_initial, sphTDSE.cpp:119-163).  HDF5 is not available here, so the same
datasets go into a numpy .npz archive: /nr, /mr, /nl, /nm, /m0, /rmin, /rmax and /coef1
(complex128 [m][l][r], the layout of coefficient<dims_t>).
"""
import numpy as np


def save_state(path, coef, n_r, p, n_l, n_m, m0, rmin, rmax):
    c = np.ascontiguousarray(coef, dtype=np.complex128).reshape(n_m, n_l, n_r)
    np.savez(path, nr=np.uint64(n_r), mr=np.uint64(p), nl=np.uint64(n_l), nm=np.uint64(n_m), m0=np.int64(m0),
             rmin=np.float64(rmin), rmax=np.float64(rmax), coef1=c)


def load_initial(path, n_r, p, n_l, n_m, m0, rmin, rmax):
    """(status, coef[n_m][n_l][n_r]) with init::load_initial's checks and codes: -1 different
    radial grid (n_r, rmin, rmax), -2 different B-spline degree, -3 the file's m range is not
    inside this grid's, -4 more l channels than this grid has; 0 on success, the file's
    channels placed at their m and the rest zero."""
    f = np.load(path)
    nr, mr, nl, nm, fm0 = int(f["nr"]), int(f["mr"]), int(f["nl"]), int(f["nm"]), int(f["m0"])
    if nr != n_r or float(f["rmin"]) != rmin or float(f["rmax"]) != rmax:
        return -1, None
    if mr != p:
        return -2, None
    if fm0 < m0 or fm0 + nm > m0 + n_m:
        return -3, None
    if nl > n_l:
        return -4, None
    out = np.zeros((n_m, n_l, n_r), np.complex128)
    src = np.asarray(f["coef1"]).reshape(nm, nl, nr)
    out[fm0 - m0: fm0 - m0 + nm, :nl, :] = src
    return 0, out
