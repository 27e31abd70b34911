"""Momentum spectra on the CPU: the special functions against independent implementations
(mpmath, scipy), the product's host tables (qpc_pcs_tables, qpc_tsurff_tables) and the numpy
oracle (oracle/momentum_oracle.py) against the reference's own outputs (tests/golden/pcs_*.npz,
tsurff_*.npz, made by tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import golden, rel_l2
from oracle import momentum_oracle as mo


def test_coulomb_f_against_mpmath(q):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 30
    worst = 0.0
    for eta in (0.0, -0.5, -2.0, -10.0, 1.5):
        for rho in (1e-3, 0.3, 0.99, 2.5, 20.0, 150.0):
            F, Fp = q.coulomb_f(eta, rho, 12)
            for l in (0, 1, 4, 12):
                f = float(mp.coulombf(l, eta, rho))
                fp = float(mp.diff(lambda x: mp.coulombf(l, eta, x), rho))
                worst = max(worst, max(abs(F[l] - f), abs(Fp[l] - fp)) / max(abs(f), abs(fp)))
    assert worst < 1e-12, worst


def test_coulomb_sigma_against_mpmath(q):
    mp = pytest.importorskip("mpmath")
    for eta in (-0.3, -4.0, -40.0, 2.0):
        s = q.coulomb_sigma(eta, 6)
        ref = np.array([float(mp.arg(mp.gamma(l + 1 + 1j * eta))) for l in range(7)])
        d = (s - ref + np.pi) % (2 * np.pi) - np.pi
        assert np.abs(d).max() < 1e-13


def test_sph_legendre_against_scipy(q):
    sp = pytest.importorskip("scipy.special")
    from math import factorial
    for x in (-0.93, 0.0, 0.41, 1.0):
        y = q.sph_legendre(9, x)
        for l in range(10):
            for m in range(l + 1):
                ref = np.sqrt((2 * l + 1) / (4 * np.pi) * factorial(l - m) / factorial(l + m)) * sp.lpmv(m, l, x)
                assert abs(y[l * (l + 1) // 2 + m] - ref) < 1e-13 * max(1.0, abs(ref))


@pytest.mark.parametrize("tag", ["pcs_small", "pcs_ep"])
@pytest.mark.parametrize("case", ["coul", "plane"])
def test_pcs_tables_match_reference(q, tag, case):
    g = golden(tag)
    n_r, p, n_l, n_m, m0 = (int(g[k]) for k in ("n_r", "p", "n_l", "n_m", "m0"))
    kmin, kmax, t0, t1, p0, p1, zc, rb, flag = g[case + "_grid"]
    kn = q.linear_knots(n_r, p, 0.0, float(g["rmax"]))
    t = q.pcs_tables(n_r, p, n_l, kn, int(g["nkr"]), int(g["nkt"]), int(g["nkp"]), kmin, kmax, t0, t1, p0, p1, zc, rb, int(flag), n_m, m0)
    for k in ("kr", "kt", "kp", "plm", "exm", "cps"):
        assert np.abs(t[k] - g[case + "_" + k]).max() < 1e-13, k
    ijl = g[case + "_ijl"]
    assert np.abs(t["ijl"] - ijl).max() < 1e-13 * np.abs(ijl).max()


@pytest.mark.parametrize("tag", ["pcs_small", "pcs_ep"])
@pytest.mark.parametrize("case", ["coul", "plane"])
def test_pcs_oracle_matches_reference(tag, case):
    g = golden(tag)
    t = {k: g[case + "_" + k] for k in ("kr", "ijl", "plm", "exm", "cps")}
    lmd, pmd, pad = mo.pcs_measure(t, g["coef"], int(g["m0"]))
    assert rel_l2(lmd, g[case + "_lmd"]) < 1e-13
    assert rel_l2(pmd, g[case + "_pmd"]) < 1e-13
    assert rel_l2(pad, g[case + "_pad"]) < 1e-13


@pytest.mark.parametrize("tag", ["tsurff_small", "tsurff_ep"])
def test_tsurff_tables_match_reference(q, tag):
    g = golden(tag)
    n_r, p, n_l, n_m, m0 = (int(g[k]) for k in ("n_r", "p", "n_l", "n_m", "m0"))
    kmin, kmax, t0, t1, p0, p1, flag = g["grid"]
    t = q.tsurff_tables(n_r, p, n_l, g["knots"], float(g["r0"]), float(g["tzc"]), int(g["nkr"]), int(g["nkt"]), int(g["nkp"]),
                        kmin, kmax, t0, t1, p0, p1, int(flag), n_m, m0)
    assert np.array_equal(t["ib"], g["ib"])
    for k in ("kr", "kt", "kp", "b0", "br", "y0", "e0", "pmat"):
        assert np.abs(t[k] - g[k]).max() < 1e-13 * max(1.0, np.abs(g[k]).max()), k
    for k in ("j0", "jr"):
        assert np.abs(t[k] - g[k]).max() < 1e-12 * np.abs(g[k]).max(), k


def _tables(g):
    return {k: g[k] for k in ("kr", "kt", "kp", "ib", "b0", "br", "j0", "jr", "y0", "e0", "pmat")}


def test_tsurff_oracle_z_loop_matches_reference(oracle):
    """the length-gauge driver loop with t-SURFF: oracle CN step + oracle accumulate per step"""
    g = golden("tsurff_small")
    n_l, dt, nt, nfree = int(g["n_l"]), float(g["dt"]), int(g["nt"]), int(g["nfree"])
    og = oracle.grid(g["S"], g["R"], g["H"], dt, n_l)
    ts = mo.Tsurff(_tables(g), n_l, 1, 0)
    c = g["init"].reshape(1, -1)
    f = g["field"]
    for it in range(nt + nfree):
        if it < nt:
            c = oracle.step(og, c, f[it], f[it + 1])
            ts.accumulate(c.reshape(1, n_l, -1), dt, (f[it], f[it + 1]))
        else:
            c = oracle.step(og, c)
            ts.accumulate(c.reshape(1, n_l, -1), dt)
    assert rel_l2(c.reshape(g["coef"].shape), g["coef"]) < 1e-12
    assert np.abs(ts.clock - g["clock"]).max() < 1e-14
    assert rel_l2(ts.work, g["work"]) < 1e-11


def test_tsurff_oracle_xy_loop_matches_reference(voracle):
    """the velocity-gauge elliptical driver loop with t-SURFF (sphTDSE.cpp:936-945)"""
    g = golden("tsurff_ep")
    n_l, n_m, m0, dt, nt, nfree = int(g["n_l"]), int(g["n_m"]), int(g["m0"]), float(g["dt"]), int(g["nt"]), int(g["nfree"])
    vg = voracle.grid(g["S"], g["RINV"], g["D"], g["H"], dt, n_l, n_m, m0)
    ts = mo.Tsurff(_tables(g), n_l, n_m, m0)
    c = g["init"].reshape(1, n_m, n_l, -1)
    a = g["field"]
    for it in range(nt + nfree):
        if it < nt:
            c = voracle.run(vg, c, a[None, it:it + 2], 1, 1)
            ts.accumulate(c[0], dt, (a[it, 0], a[it + 1, 0], a[it, 1], a[it + 1, 1]))
        else:
            c = voracle.run(vg, c, a[None, :2] * 0, 0, 1)
            ts.accumulate(c[0], dt)
    assert rel_l2(c[0], g["coef"]) < 1e-12
    assert np.abs(ts.clock - g["clock"]).max() < 1e-14
    assert rel_l2(ts.work, g["work"]) < 1e-11


def test_table_arguments_are_checked(q):
    kn = q.linear_knots(64, 6, 0.0, 30.0)
    with pytest.raises(q.QpcError):
        q.pcs_tables(64, 6, 6, kn, 4, 2, 2, 0.0, 1.0, 0, 3, 0, 6, 1.0)      # |k| = 0 on the grid
    with pytest.raises(q.QpcError):
        q.tsurff_tables(64, 6, 6, kn, 31.0, 0.0, 4, 2, 2, 0.1, 1.0, 0, 3, 0, 6)  # surface outside the box
    with pytest.raises(q.QpcError):
        q.coulomb_f(-1.0, 0.0, 3)


def test_pcs_numeric_tables_match_reference(q):
    """numerical partial waves of V = -(1 + 17 e^{-2r})/r: both sides integrate the radial equation
    to a relative tolerance of 5e-11 (different Runge-Kutta pairs), so they agree to ~1e-9"""
    g = golden("pcsnum_small")
    kmin, kmax, t0, t1, p0, p1, flag = g["grid"]
    kn = q.linear_knots(int(g["n_r"]), int(g["p"]), 0.0, float(g["rmax"]))
    t = q.pcs_tables_numeric(int(g["n_r"]), int(g["p"]), int(g["n_l"]), kn, int(g["nkr"]), int(g["nkt"]), int(g["nkp"]),
                             kmin, kmax, t0, t1, p0, p1, (q.POTENTIAL_YUKAWA, float(g["zc"]), float(g["zs"]), float(g["sigma"])), int(flag))
    assert np.abs(t["cps"] - g["cps"]).max() < 1e-9
    prod, ref = t["ijl"] * t["cps"][:, :, None], g["ijl"] * g["cps"][:, :, None]
    assert np.abs(prod - ref).max() < 1e-8 * np.abs(ref).max()


def test_pcs_numeric_oracle_matches_reference(q):
    g = golden("pcsnum_small")
    kn = q.linear_knots(int(g["n_r"]), int(g["p"]), 0.0, float(g["rmax"]))
    kmin, kmax, t0, t1, p0, p1, flag = g["grid"]
    ang = q.pcs_tables(int(g["n_r"]), int(g["p"]), int(g["n_l"]), kn, int(g["nkr"]), int(g["nkt"]), int(g["nkp"]), kmin, kmax,
                       t0, t1, p0, p1, 1.0)
    t = {"kr": g["kr"], "ijl": g["ijl"], "cps": g["cps"], "plm": ang["plm"], "exm": ang["exm"]}
    lmd, pmd, _ = mo.pcs_measure(t, g["coef"], 0)
    assert rel_l2(lmd, g["lmd"]) < 1e-13
    assert rel_l2(pmd, g["pmd"]) < 1e-13
