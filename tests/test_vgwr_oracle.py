"""Velocity-gauge elliptical propagator: the engine's angular eigensystems and the CPU
oracle (oracle/oracle_cn.cpp) against the reference's propagator_cn_hc_vgwr run through
oracle/_ref (tests/golden/vgwr_*.npz)."""
import numpy as np
import pytest

from conftest import band_mask, golden, rel_l2

CASES = ["vgwr_ep", "vgwr_ep6"]


@pytest.mark.parametrize("tag", CASES)
def test_angular_eigenvalues_match_reference(q, tag):
    g = golden(tag)
    n_l, n_m, m0 = int(g["n_l"]), int(g["n_m"]), int(g["m0"])
    for c in range(4):
        lam, P = q.vgwr_angular(n_l, n_m, m0, c)
        assert np.abs(np.sort(lam) - np.sort(g["zeig"][c])).max() < 1e-13
        assert np.abs(P @ P.conj().T - np.eye(lam.size)).max() < 1e-13


@pytest.mark.parametrize("tag", CASES)
def test_setup_matches_reference(q, tag):
    g = golden(tag)
    n_r, p = int(g["n_r"]), int(g["p"])
    nlh = g["H"].shape[0]
    S, R, Ri, D, H = q.radial_setup(n_r, p, nlh, q.linear_knots(n_r, p, 0.0, float(g["rmax"])))
    mask = band_mask(n_r, p)   # entries past the last row are padding, unused by either side
    for a, b in ((S, g["S"]), (Ri, g["RINV"]), (D, g["D"]), (H, g["H"])):
        a, b = a * mask, b * mask
        assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()


@pytest.mark.parametrize("tag", CASES)
def test_oracle_matches_reference(voracle, tag):
    g = golden(tag)
    og = voracle.grid(g["S"], g["RINV"], g["D"], g["H"], float(g["dt"]), int(g["n_l"]), int(g["n_m"]), int(g["m0"]))
    nt, nf = int(g["nt"]), int(g["nfree"])
    c = voracle.run(og, g["init"].reshape(1, -1), g["atab"][None], [nt], [nt + nf])
    assert rel_l2(c.reshape(g["coef"].shape), g["coef"]) < 1e-12


def vgwr_states(voracle, g, R=None):
    """the oracle's state before every step of the golden run (the driver's observation points)"""
    og = voracle.grid(g["S"], g["RINV"], g["D"], g["H"], float(g["dt"]), int(g["n_l"]), int(g["n_m"]), int(g["m0"]))
    nt, nf = int(g["nt"]), int(g["nfree"])
    c = g["init"].reshape(1, -1)
    out = []
    for s in range(nt + nf):
        out.append(c[0].copy())
        if s < nt:
            c = voracle.run(og, c, g["atab"][None, s:s + 2], [1], [1])
        else:
            c = voracle.run(og, c, g["atab"][None, :2], [0], [1])
    return out


@pytest.mark.parametrize("tag", CASES)
def test_dipole_oracle_matches_reference(q, voracle, tag):
    """observable_r restated (oracle/observable_oracle.py) on the oracle's states against the
    reference's <x>, <y> before every step of the golden run."""
    import sys, os
    from conftest import ROOT
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import observable_oracle as oo
    g = golden(tag)
    n_r, p, n_l, n_m, m0 = int(g["n_r"]), int(g["p"]), int(g["n_l"]), int(g["n_m"]), int(g["m0"])
    _, R, _, _, _ = q.radial_setup(n_r, p, 1, q.linear_knots(n_r, p, 0.0, float(g["rmax"])))
    xs, ys = [], []
    for c in vgwr_states(voracle, g):
        x, y = oo.dipole_xy(c, R, n_l, n_m, m0)
        xs.append(x)
        ys.append(y)
    scale = np.abs(np.concatenate([g["xlist"], g["ylist"]])).max()
    assert np.abs(np.array(xs) - g["xlist"]).max() < 1e-12 * scale
    assert np.abs(np.array(ys) - g["ylist"]).max() < 1e-12 * scale
