"""Momentum spectra on the GPU against the reference's outputs (tests/golden/pcs_*.npz,
tsurff_*.npz) and the CPU oracle (oracle/momentum_oracle.py): the PCS projections
measure_lmd / measure_prj / measure_pad, and t-SURFF accumulated inside the driver loops
of the length-gauge and the velocity-gauge elliptical propagators."""
import numpy as np
import pytest

from conftest import golden, rel_l2
from oracle import momentum_oracle as mo

pytestmark = pytest.mark.gpu


def _pcs_from_golden(q, g, case):
    n_r, p, n_l, n_m, m0 = (int(g[k]) for k in ("n_r", "p", "n_l", "n_m", "m0"))
    kmin, kmax, t0, t1, p0, p1, zc, rb, flag = g[case + "_grid"]
    kn = q.linear_knots(n_r, p, 0.0, float(g["rmax"]))
    return q.spectrum_c_pcs(int(g["nkr"]), int(g["nkt"]), int(g["nkp"])).initialize(
        n_r, p, n_l, kn, kmin, kmax, t0, t1, p0, p1, zc, rb, int(flag), n_m, m0)


@pytest.mark.parametrize("tag", ["pcs_small", "pcs_ep"])
@pytest.mark.parametrize("case", ["coul", "plane"])
def test_pcs_matches_reference(q, tag, case):
    g = golden(tag)
    pcs = _pcs_from_golden(q, g, case)
    c = g["coef"][None]
    assert rel_l2(pcs.measure_lmd(c)[0], g[case + "_lmd"]) < 1e-12
    assert rel_l2(pcs.measure_prj(c)[0], g[case + "_pmd"]) < 1e-12
    assert rel_l2(pcs.measure_pad(c)[0], g[case + "_pad"]) < 1e-12


def test_pcs_batch_against_oracle(q):
    """19 wavefunctions (not a multiple of the 8 a block projects together), more than one block
    of |k| values, on a two-m grid."""
    n_r, p, n_l, n_m, m0, B = 160, 6, 7, 2, -1, 19
    kn = q.linear_knots(n_r, p, 0.0, 80.0)
    nk = (150, 7, 3)
    pcs = q.spectrum_c_pcs(*nk).initialize(n_r, p, n_l, kn, 0.05, 2.5, 0.0, np.pi, 0.0, 4.0, 1.0, 0.0, 0, n_m, m0)
    rng = np.random.default_rng(3)
    c = (rng.standard_normal((B, n_m, n_l, n_r)) + 1j * rng.standard_normal((B, n_m, n_l, n_r))) * np.exp(-np.arange(n_r) / 30.0)
    lmd, pmd, pad = pcs.measure_lmd(c), pcs.measure_prj(c), pcs.measure_pad(c)
    for i in (0, 7, 8, 18):
        ol, op, oa = mo.pcs_measure(pcs.tables, c[i], m0)
        assert rel_l2(lmd[i], ol) < 1e-12
        assert rel_l2(pmd[i], op) < 1e-12
        assert rel_l2(pad[i], oa) < 1e-12


def test_pcs_on_the_resident_state(q):
    g = golden("pcs_small")
    pcs = _pcs_from_golden(q, g, "coul")
    s = golden("small_setup")
    prop = q.propagator_cn_hc_lgwz().initialize(64, 6, 6, s["S"], s["R"], s["H"], 0.05, n_inst=3)
    rng = np.random.default_rng(5)
    c = rng.standard_normal((3, 1, 6, 64)) + 1j * rng.standard_normal((3, 1, 6, 64))
    prop.put(c)
    assert rel_l2(pcs.measure_prj(prop), pcs.measure_prj(c)) < 1e-15


def _tsurff(q, g, n_inst=1):
    n_r, p, n_l, n_m, m0 = (int(g[k]) for k in ("n_r", "p", "n_l", "n_m", "m0"))
    kmin, kmax, t0, t1, p0, p1, flag = g["grid"]
    return q.spectrum_c_tsf(int(g["nkr"]), int(g["nkt"]), int(g["nkp"])).initialize(
        n_r, p, n_l, g["knots"], float(g["r0"]), float(g["tzc"]), kmin, kmax, t0, t1, p0, p1, int(flag), n_m, m0, n_inst)


def test_tsurff_length_gauge_loop_matches_reference(q):
    """propagate(f_i, f_i+1) + accumulate(f_i, f_i+1, dt) per step, then field-free steps with
    accumulate(dt): the reference's driver loop with t-SURFF (sphTDSE.cpp:786-831)"""
    g = golden("tsurff_small")
    n_l, dt, nt, nfree = int(g["n_l"]), float(g["dt"]), int(g["nt"]), int(g["nfree"])
    prop = q.propagator_cn_hc_lgwz().initialize(int(g["n_r"]), int(g["p"]), n_l, g["S"], g["R"], g["H"], dt)
    prop.put(g["init"][None])
    ts = _tsurff(q, g)
    f = g["field"]
    for it in range(nt + nfree):
        if it < nt:
            prop.propagate(f[it], f[it + 1])
            ts.accumulate(prop, dt, (f[it], f[it + 1]))
        else:
            prop.propagate()
            ts.accumulate(prop, dt)
    work, clock = ts.get()
    assert rel_l2(prop.get()[0], g["coef"]) < 1e-11
    assert np.abs(clock[0] - g["clock"]).max() < 1e-14
    assert rel_l2(work[0], g["work"]) < 1e-10


def test_tsurff_elliptical_loop_matches_reference(q):
    g = golden("tsurff_ep")
    n_r, p, n_l, n_m, m0 = (int(g[k]) for k in ("n_r", "p", "n_l", "n_m", "m0"))
    dt, nt, nfree = float(g["dt"]), int(g["nt"]), int(g["nfree"])
    prop = q.propagator_cn_hc_vgwr().initialize(n_r, p, n_l, n_m, m0, g["S"], g["RINV"], g["D"], g["H"], dt)
    prop.put(g["init"][None])
    ts = _tsurff(q, g)
    a = g["field"]
    for it in range(nt + nfree):
        if it < nt:
            prop.propagate(a[it, 0], a[it + 1, 0], a[it, 1], a[it + 1, 1])
            ts.accumulate(prop, dt, (a[it, 0], a[it + 1, 0], a[it, 1], a[it + 1, 1]))
        else:
            prop.propagate()
            ts.accumulate(prop, dt)
    work, clock = ts.get()
    assert rel_l2(prop.get()[0], g["coef"]) < 1e-11
    assert np.abs(clock[0] - g["clock"]).max() < 1e-14
    assert rel_l2(work[0], g["work"]) < 1e-10


@pytest.mark.parametrize("mode", ["free", "z", "xy"])
def test_tsurff_batch_against_oracle(q, mode):
    """three wavefunctions with their own field values, host arrays in, every accumulate form"""
    g = golden("tsurff_ep")
    n_l, n_m, m0, B, dt = int(g["n_l"]), int(g["n_m"]), int(g["m0"]), 3, 0.05
    ts = _tsurff(q, g, n_inst=B)
    ors = [mo.Tsurff(ts.tables, n_l, n_m, m0) for _ in range(B)]
    rng = np.random.default_rng(7)
    for step in range(6):
        c = (rng.standard_normal((B,) + g["init"].shape) + 1j * rng.standard_normal((B,) + g["init"].shape)) * 0.1
        a = None if mode == "free" else rng.uniform(-0.5, 0.5, (B, 2 if mode == "z" else 4))
        ts.accumulate(c, dt, a)
        for i in range(B):
            ors[i].accumulate(c[i], dt, None if a is None else tuple(a[i]))
    work, clock = ts.get()
    for i in range(B):
        assert rel_l2(work[i], ors[i].work) < 1e-12
        assert np.abs(clock[i] - ors[i].clock).max() < 1e-15
    ts.clearwork()
    work, clock = ts.get()
    assert not work.any() and not clock.any()


def test_pcs_numeric_partial_waves_match_reference(q):
    """the numerical PCS for a screened potential (ODE-tolerance-limited agreement, ~1e-9)"""
    g = golden("pcsnum_small")
    kmin, kmax, t0, t1, p0, p1, flag = g["grid"]
    kn = q.linear_knots(int(g["n_r"]), int(g["p"]), 0.0, float(g["rmax"]))
    pcs = q.spectrum_c_pcs(int(g["nkr"]), int(g["nkt"]), int(g["nkp"])).initialize(
        int(g["n_r"]), int(g["p"]), int(g["n_l"]), kn, kmin, kmax, t0, t1, p0, p1, 1.0, flag=int(flag),
        potential=(q.POTENTIAL_YUKAWA, float(g["zc"]), float(g["zs"]), float(g["sigma"])))
    c = g["coef"][None]
    assert rel_l2(pcs.measure_lmd(c)[0], g["lmd"]) < 1e-8
    assert rel_l2(pcs.measure_prj(c)[0], g["pmd"]) < 1e-8
