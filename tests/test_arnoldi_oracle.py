"""The Arnoldi oracle (oracle/oracle_arnoldi.cpp) against the reference's own
propagator_hc_lgwz (la_1e.hpp), run through oracle/_ref and stored as golden
fixtures, and the engine's host Cholesky against operator_sc::cholesky()."""
import numpy as np
import pytest

from conftest import golden, rel_l2


def _small_grid(aoracle, H=None, dt=0.1):
    s = golden("small_setup")
    a = golden("arnoldi_small")
    return aoracle.grid(s["S"], s["R"], s["H"] if H is None else H, s["y10"], dt, int(s["n_l"]),
                        kmax=int(a["kmax"]), emin=float(a["emin"]), emax=float(a["emax"]))


def test_cholesky_matches_reference(q, aoracle):
    s = golden("small_setup")
    ref = golden("arnoldi_small")["chol"]
    assert np.abs(aoracle.chol(s["S"]) - ref).max() <= 1e-14 * np.abs(ref).max()
    assert np.abs(q.cholesky_band(s["S"], int(s["p"])) - ref).max() <= 1e-14 * np.abs(ref).max()


def test_cholesky_rejects_indefinite(q):
    S = np.zeros((20, 3))
    S[:, 0] = 1.0
    S[7, 0] = -1.0
    with pytest.raises(q.QpcError):
        q.cholesky_band(S, 2)


def test_oracle_converged_run(aoracle):
    """3000 steps of dt = 0.01 from the ground state (the expansion converges,
    criterion 2 in every step): the oracle reproduces the reference's coefficients
    and its criterion codes."""
    s, a = golden("small_setup"), golden("arnoldi_small")
    g = _small_grid(aoracle, dt=float(a["conv_dt"]))
    c, crit, ms = aoracle.run(g, s["gs_coef"].reshape(1, -1), a["conv_ez"])
    assert rel_l2(c.reshape(a["conv_coef"].shape), a["conv_coef"]) < 1e-11
    assert np.array_equal(crit[0], a["conv_crit"])


@pytest.mark.parametrize("tag", ["step1", "step3"])
def test_oracle_steps(aoracle, tag):
    a = golden("arnoldi_small")
    g = _small_grid(aoracle, dt=float(a[tag + "_dt"]))
    c, crit, ms = aoracle.run(g, a["conv_coef"].reshape(1, -1), a[tag + "_ez"])
    assert rel_l2(c.reshape(a[tag + "_coef"].shape), a[tag + "_coef"]) < 1e-12
    assert np.array_equal(crit[0], a[tag + "_crit"])


def test_oracle_yukawa_step(aoracle):
    a = golden("arnoldi_small")
    g = _small_grid(aoracle, H=golden("small_yukawa")["H"], dt=float(a["ystep1_dt"]))
    c, crit, _ = aoracle.run(g, a["conv_coef"].reshape(1, -1), a["ystep1_ez"])
    assert rel_l2(c.reshape(a["ystep1_coef"].shape), a["ystep1_coef"]) < 1e-12


def test_oracle_breakdown(aoracle):
    """Field-free steps of an eigenstate: the expansion stops at m = 1 (<v|S|v> < 1e-13)
    and the step is the phase exp(-i dt E)."""
    s, a = golden("small_setup"), golden("arnoldi_small")
    g = _small_grid(aoracle, dt=float(a["bd_dt"]))
    c, crit, ms = aoracle.run(g, s["gs_coef"].reshape(1, -1), a["bd_ez"])
    assert rel_l2(c.reshape(a["bd_coef"].shape), a["bd_coef"]) < 1e-13
    assert np.all(ms == 1) and np.array_equal(crit[0], a["bd_crit"])
    e = float(s["gs_energy"][0])
    ph = np.exp(-1j * e * float(a["bd_dt"]) * a["bd_ez"].size)
    assert rel_l2(c.reshape(s["gs_coef"].shape), ph * s["gs_coef"]) < 1e-9


@pytest.mark.parametrize("tag", ["step1", "step2"])
def test_oracle_mid_steps(aoracle, tag):
    m, a = golden("mid_pulse"), golden("arnoldi_mid")
    from conftest import engine
    q = engine()
    n_r, p, n_l, rmax = int(m["n_r"]), int(m["p"]), int(m["n_l"]), float(m["rmax"])
    kn = q.linear_knots(n_r, p, 0.0, rmax)
    S, R, _, _, H = q.radial_setup(n_r, p, n_l, kn)
    g = aoracle.grid(S, R, H, q.y10_coupling(n_l), float(a[tag + "_dt"]), n_l, kmax=int(a["kmax"]))
    c, crit, _ = aoracle.run(g, a["init"].reshape(1, -1), a[tag + "_ez"])
    assert rel_l2(c.reshape(a[tag + "_coef"].shape), a[tag + "_coef"]) < 1e-11
    assert np.array_equal(crit[0], a[tag + "_crit"])
