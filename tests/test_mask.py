"""Absorbing mask (absorber_mask, absorber.hpp:40-63): the engine's mask band and the CPU
oracle against the reference's own output (tests/golden/small_mask.npz)."""
import numpy as np

from conftest import band_mask, golden, rel_l2


def test_mask_band_matches_reference(q):
    s, m = golden("small_setup"), golden("small_mask")
    n_r, p = int(s["n_r"]), int(s["p"])
    M = q.mask_band(n_r, p, q.linear_knots(n_r, p, 0.0, float(s["rmax"])), float(m["rmin"]), float(m["rmax_mask"]), float(m["index"]))
    bm = band_mask(n_r, p)
    assert np.abs((M - m["band"]) * bm).max() <= 1e-14 * np.abs(m["band"]).max()


def test_oracle_mask_matches_reference(aoracle):
    s, m = golden("small_setup"), golden("small_mask")
    chol = golden("arnoldi_small")["chol"]
    c = aoracle.mask(m["band"], chol, m["init"].reshape(-1), int(s["n_l"]))
    assert rel_l2(c.reshape(m["coef"].shape), m["coef"]) < 1e-13
