"""Parity of the GPU velocity-gauge elliptical propagator (propagator_cn_hc_vgwr, through
the C ABI) against the reference's golden vectors and the CPU oracle; 1e-12 relative L2
for these short runs (the bar for full pulses is 1e-10)."""
import numpy as np
import pytest

from conftest import golden, rel_l2

pytestmark = pytest.mark.gpu

CASES = ["vgwr_ep", "vgwr_ep6"]


def make(q, g, n_inst=1):
    return q.propagator_cn_hc_vgwr().initialize(int(g["n_r"]), int(g["p"]), int(g["n_l"]), int(g["n_m"]), int(g["m0"]),
                                               g["S"], g["RINV"], g["D"], g["H"], float(g["dt"]), n_inst=n_inst)


@pytest.mark.parametrize("tag", CASES)
def test_golden_run(q, tag):
    g = golden(tag)
    pr = make(q, g)
    pr.put(g["init"][None])
    nt, nf = int(g["nt"]), int(g["nfree"])
    pr.run(g["atab"][None], [nt], [nt + nf])
    assert rel_l2(pr.get()[0], g["coef"]) < 1e-12
    assert abs(pr.norm()[0] - g["norm"][0]) < 1e-12 * g["norm"][0]


@pytest.mark.parametrize("tag", CASES)
def test_stepwise_equals_run(q, tag):
    g = golden(tag)
    pr = make(q, g)
    pr.put(g["init"][None])
    a = g["atab"]
    for s in range(int(g["nt"])):
        pr.propagate(a[s, 0], a[s + 1, 0], a[s, 1], a[s + 1, 1])
    for _ in range(int(g["nfree"])):
        pr.propagate()
    assert rel_l2(pr.get()[0], g["coef"]) < 1e-12


def test_uneven_batch_matches_oracle(q, voracle):
    g = golden("vgwr_ep6")
    B = 3
    rng = np.random.default_rng(9)
    c0 = np.stack([g["init"] * np.exp(0.3j * k) for k in range(B)])
    nt = 12
    t = 0.05 * np.arange(nt + 1)
    atab = np.stack([np.stack([0.2 * (k + 1) * np.sin(0.4 * t + k), 0.1 * np.cos(0.7 * t - k)], 1) for k in range(B)])
    nf = np.array([12, 5, 0])
    ntt = np.array([14, 12, 3])
    pr = make(q, g, B)
    pr.put(c0)
    pr.run(atab, nf, ntt)
    og = voracle.grid(g["S"], g["RINV"], g["D"], g["H"], float(g["dt"]), int(g["n_l"]), int(g["n_m"]), int(g["m0"]), B)
    ref = voracle.run(og, c0.reshape(B, -1), atab, nf, ntt)
    out = pr.get().reshape(B, -1)
    for k in range(B):
        assert rel_l2(out[k], ref[k]) < 1e-12, k


def test_mid_grid_matches_oracle(q, voracle):
    """A mid-size grid (n_m = 21, m0 = -10, n_l = 21: 441 channels, parity blocks of 220 and 221;
    N_r = 200, p = 6): the transforms run as the library's own GEMM kernels on sizes that are no
    multiple of their tiles, with the device eigensystems at that size, against the oracle's
    dense transforms, 6 field steps and 2 field-free ones."""
    n_r, p, n_l, n_m, m0, dt = 200, 6, 21, 21, -10, 0.05
    nlh = max(abs(m0), abs(m0 + n_m - 1)) + n_l
    S, _, Ri, D, H = q.radial_setup(n_r, p, nlh, q.linear_knots(n_r, p, 0.0, 100.0))
    rng = np.random.default_rng(31)
    r = np.arange(n_r)
    c0 = (rng.standard_normal((1, n_m, n_l, n_r)) + 1j * rng.standard_normal((1, n_m, n_l, n_r))) * np.exp(-r / 25.0)
    nt = 6
    t = dt * np.arange(nt + 1)
    atab = np.stack([0.4 * np.sin(0.3 * t + 0.2), 0.25 * np.cos(0.3 * t)], 1)[None]
    pr = q.propagator_cn_hc_vgwr().initialize(n_r, p, n_l, n_m, m0, S, Ri, D, H, dt)
    pr.put(c0)
    n0 = pr.norm()[0]
    pr.run(atab, [nt], [nt + 2])
    got = pr.get().reshape(-1)
    og = voracle.grid(S, Ri, D, H, dt, n_l, n_m, m0)
    ref = voracle.run(og, c0.reshape(1, -1), atab, [nt], [nt + 2])
    assert rel_l2(got, ref[0]) < 1e-12
    assert abs(pr.norm()[0] - n0) < 1e-12 * n0


@pytest.mark.parametrize("tag", CASES)
def test_golden_dipole_list(q, tag):
    """<x>, <y> before every step (observable_r inside the device loop) against the reference's
    record of the same run, and the final state unchanged by the observation."""
    g = golden(tag)
    n_r, p = int(g["n_r"]), int(g["p"])
    _, R, _, _, _ = q.radial_setup(n_r, p, 1, q.linear_knots(n_r, p, 0.0, float(g["rmax"])))
    pr = make(q, g)
    pr.put(g["init"][None])
    nt, nf = int(g["nt"]), int(g["nfree"])
    x, y = pr.run_dipole(g["atab"][None], [nt], [nt + nf], R)
    scale = np.abs(np.concatenate([g["xlist"], g["ylist"]])).max()
    assert np.abs(x[0] - g["xlist"]).max() < 1e-12 * scale
    assert np.abs(y[0] - g["ylist"]).max() < 1e-12 * scale
    assert rel_l2(pr.get()[0], g["coef"]) < 1e-12


def test_dipole_list_uneven_batch(q, voracle):
    """three instances with their own fields and step counts: each instance's <x>, <y> list against
    the numpy restatement of observable_r on the oracle's states"""
    import os
    import sys
    from conftest import ROOT
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import observable_oracle as oo
    g = golden("vgwr_ep6")
    n_r, p, n_l, n_m, m0 = int(g["n_r"]), int(g["p"]), int(g["n_l"]), int(g["n_m"]), int(g["m0"])
    _, R, _, _, _ = q.radial_setup(n_r, p, 1, q.linear_knots(n_r, p, 0.0, float(g["rmax"])))
    B = 3
    c0 = np.stack([g["init"] * np.exp(0.3j * k) * (1.0 + 0.1 * k) for k in range(B)])
    nt = 10
    t = 0.05 * np.arange(nt + 1)
    atab = np.stack([np.stack([0.2 * (k + 1) * np.sin(0.4 * t + k), 0.1 * np.cos(0.7 * t - k)], 1) for k in range(B)])
    nf = np.array([10, 4, 0])
    ntt = np.array([12, 9, 3])
    pr = make(q, g, B)
    pr.put(c0)
    x, y = pr.run_dipole(atab, nf, ntt, R)
    og = voracle.grid(g["S"], g["RINV"], g["D"], g["H"], float(g["dt"]), n_l, n_m, m0)
    for k in range(B):
        c = c0[k].reshape(1, -1)
        for s in range(ntt[k]):
            xr, yr = oo.dipole_xy(c[0], R, n_l, n_m, m0)
            sc = max(abs(xr), abs(yr), 1e-300)
            assert abs(x[k, s] - xr) < 1e-12 * sc and abs(y[k, s] - yr) < 1e-12 * sc, (k, s)
            c = voracle.run(og, c, atab[k:k + 1, s:s + 2] if s < nf[k] else atab[k:k + 1, :2], [1 if s < nf[k] else 0], [1])
        assert np.all(x[k, ntt[k]:] == 0.0)
