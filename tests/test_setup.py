"""Host setup of the engine (qpc_setup.cpp through the C ABI) against the
reference's own matrices (tests/golden/*)."""
import numpy as np

from conftest import band_mask, golden, rel_l2


def _small(q):
    g = golden("small_setup")
    n_r, p, n_l = int(g["n_r"]), int(g["p"]), int(g["n_l"])
    t = q.linear_knots(n_r, p, 0.0, float(g["rmax"]))
    return g, n_r, p, n_l, t


def test_knots(q):
    g, n_r, p, n_l, t = _small(q)
    assert np.array_equal(t, g["knots"])


def test_radial_matrices(q):
    g, n_r, p, n_l, t = _small(q)
    S, R, Ri, D, H = q.radial_setup(n_r, p, n_l, t)
    m = band_mask(n_r, p)
    for a, name in ((S, "S"), (R, "R"), (Ri, "RINV"), (D, "D")):
        b = g[name]
        assert np.abs(a[m] - b[m]).max() <= 1e-14 * np.abs(b).max(), name
        assert np.all(a[~m] == 0.0)
    assert np.abs(H[:, m] - g["H"][:, m]).max() <= 1e-13 * np.abs(g["H"]).max()


def test_yukawa_potential(q):
    g, n_r, p, n_l, t = _small(q)
    y = golden("small_yukawa")
    _, _, _, _, H = q.radial_setup(n_r, p, n_l, t, (q.POTENTIAL_YUKAWA, 1.0, 17.0, 2.0))
    m = band_mask(n_r, p)
    assert np.abs(H[:, m] - y["H"][:, m]).max() <= 1e-13 * np.abs(y["H"]).max()


def test_y10_eigensystem(q):
    g, n_r, p, n_l, t = _small(q)
    lam, P = q.y10_eigen(n_l, 0)
    assert np.abs(lam - g["yeig"]).max() < 1e-15
    # the decomposition P^T diag(lam) P is what the step uses; row order and signs are free
    A = P.T @ np.diag(lam) @ P
    Ar = g["yprj"].T @ np.diag(g["yeig"]) @ g["yprj"]
    assert np.abs(A - Ar).max() < 1e-14
    assert np.abs(P @ P.T - np.eye(n_l)).max() < 1e-14
    # pair structure the engine relies on: v(-s) = D v(s), exact
    D = np.diag((-1.0) ** np.arange(n_l))
    for k in range(n_l // 2):
        assert np.array_equal(P[k], D @ P[n_l - 1 - k])


def test_y10_eigensystem_odd_and_m(q):
    for n_l, m in ((7, 0), (21, 0), (9, 3), (8, -2)):
        lam, P = q.y10_eigen(n_l, m)
        y = q.y10_coupling(n_l, m)
        T = np.diag(y[:-1], 1) + np.diag(y[:-1], -1)
        assert np.abs(P.T @ np.diag(lam) @ P - T).max() < 1e-14
        if n_l % 2:
            assert lam[n_l // 2] == 0.0 and np.all(P[n_l // 2][1::2] == 0.0)


def test_ground_state(q):
    g, n_r, p, n_l, t = _small(q)
    S, R, _, _, H = q.radial_setup(n_r, p, n_l, t)
    c, e = q.ground_state(S, H, n_l)
    assert abs(e - g["gs_energy"][0]) < 1e-13
    assert abs(e + 0.5) < 1e-6  # hydrogen 1s
    ref = g["gs_coef"]
    assert min(rel_l2(c[0], ref), rel_l2(-c[0], ref)) < 1e-12
    y = golden("small_yukawa")
    _, _, _, _, Hy = q.radial_setup(n_r, p, n_l, t, (q.POTENTIAL_YUKAWA, 1.0, 17.0, 2.0))
    cy, ey = q.ground_state(S, Hy, n_l)
    assert abs(ey - y["gs_energy"][0]) < 1e-12 * abs(ey)


def test_cn_factorisation_matches_lu_zsb(q):
    g, n_r, p, n_l, t = _small(q)
    dt = float(g["dt"])
    for l in range(n_l):
        Lrow, Dinv, bad = q.ldlt_csym(g["S"], g["H"][l], dt * 0.5)
        assert bad == 0
        lo = g["lower"][l]
        assert np.abs(1.0 / Dinv - lo[:, 0]).max() < 1e-14 * np.abs(lo[:, 0]).max()
        Lref = np.zeros((n_r, p), complex)
        for r in range(n_r):
            for k in range(1, p + 1):
                if r - k >= 0:
                    Lref[r, k - 1] = lo[r - k, k]
        assert np.abs(Lrow - Lref).max() < 1e-13


def test_field_table(q):
    c = golden("c0_field")
    f = q.field_sinen(float(c["e0"]), float(c["w0"]), float(c["nc"]), float(c["n0"]), float(c["cep"]), float(c["dt"]))
    assert f.size == int(c["nt"]) + 1 == 8827
    assert np.abs(f - c["f"]).max() < 1e-15
    m = golden("mid_pulse")
    fm = q.field_sinen(float(m["e0"]), float(m["w0"]), float(m["nc"]), float(m["n0"]), float(m["cep"]), float(m["dt"]))
    assert np.abs(fm - m["f"]).max() < 1e-15


def test_projection_basis(q):
    """Field-free eigenstates of the C0 grid: energies of the reference's
    eigenstate_sph (E < 2) for every l."""
    g = golden("c0_final")
    n_r, p, n_l = int(g["n_r"]), int(g["p"]), int(g["n_l"])
    t = q.linear_knots(n_r, p, 0.0, float(g["rmax"]))
    S, R, _, _, H = q.radial_setup(n_r, p, n_l, t)
    nnz = g["proj_nnz"]
    off = 0
    for l in (0, 1, 5, 20):
        e, _ = q.gen_eigen(S, H[l], 0)
        off = int(nnz[:l].sum())
        eref = g["proj_energy"][off:off + int(nnz[l])]
        assert int((e < 2.0).sum()) == nnz[l]
        assert np.abs(e[:nnz[l]] - eref).max() < 1e-10 * max(1.0, np.abs(eref).max())
