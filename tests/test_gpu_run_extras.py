"""The reference driver's per-step work inside the device loop (qpc_lgwz_run_ex): after every
propagate the t-SURFF accumulate and the absorbing mask (binsrc/sphTDSE.cpp:797-810), with no host
round trip.  Each case equals the host loop of single propagate calls with the same per-step
work, and the t-SURFF case the reference's own golden spectrum."""
import numpy as np
import pytest

from conftest import golden, rel_l2
from test_gpu_momentum import _tsurff

pytestmark = pytest.mark.gpu


def test_masked_run_matches_host_loop_and_oracle(q, oracle, aoracle):
    """20 field steps and 5 field-free ones, mask after each, one instance: the device loop against
    propagate + mask per step and against the oracle."""
    s, m = golden("small_setup"), golden("small_mask")
    n_r, p, n_l, dt = int(s["n_r"]), int(s["p"]), int(s["n_l"]), float(s["dt"])
    f = 0.05 * np.sin(0.1 * np.arange(21))
    nt, nfree = 20, 5
    run = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, s["S"], s["R"], s["H"], dt)
    run.put(m["init"][None, None])
    run.run_ex(f[None, :], [nt], [nt + nfree], mask=m["band"])
    loop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, s["S"], s["R"], s["H"], dt)
    loop.put(m["init"][None, None])
    og = oracle.grid(s["S"], s["R"], s["H"], dt, n_l)
    chol = golden("arnoldi_small")["chol"]
    c = m["init"].reshape(1, -1).copy()
    for i in range(nt + nfree):
        if i < nt:
            loop.propagate(f[i], f[i + 1])
            c = oracle.step(og, c, f[i], f[i + 1])
        else:
            loop.propagate()
            c = oracle.step(og, c)
        loop.mask(m["band"])
        c = aoracle.mask(m["band"], chol, c.reshape(-1), n_l).reshape(1, -1)
    assert rel_l2(run.get(), loop.get()) < 1e-13
    assert rel_l2(run.get().reshape(-1), c[0]) < 1e-12


def test_masked_run_uneven_batch(q, aoracle):
    """four instances with their own pulses and step counts (one field-free only) in one run,
    against each instance's own host loop"""
    s, m = golden("small_setup"), golden("small_mask")
    n_r, p, n_l, dt = int(s["n_r"]), int(s["p"]), int(s["n_l"]), float(s["dt"])
    B = 4
    rng = np.random.default_rng(12)
    c0 = np.stack([m["init"] * np.exp(0.4j * k) for k in range(B)])[:, None]
    ftab = 0.04 * np.sin(0.1 * np.arange(31)[None, :] + rng.uniform(0, 6, (B, 1)))
    nf = np.array([30, 12, 0, 7])
    ntt = np.array([33, 12, 9, 20])
    run = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, s["S"], s["R"], s["H"], dt, n_inst=B)
    run.put(c0)
    run.run_ex(ftab, nf, ntt, mask=m["band"])
    out = run.get()
    for k in range(B):
        one = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, s["S"], s["R"], s["H"], dt)
        one.put(c0[k:k + 1])
        for i in range(ntt[k]):
            if i < nf[k]:
                one.propagate(ftab[k, i], ftab[k, i + 1])
            else:
                one.propagate()
            one.mask(m["band"])
        # the batch and the single wavefunction may run different (autotuned) chain kernels
        assert rel_l2(out[k], one.get()[0]) < 1e-12, k
        one.close()


def test_tsurff_run_matches_reference(q):
    """t-SURFF accumulated inside the device loop (field steps with f(t_i), f(t_i+1), then
    field-free ones) against the reference's spectrum and clock"""
    g = golden("tsurff_small")
    n_l, dt, nt, nfree = int(g["n_l"]), float(g["dt"]), int(g["nt"]), int(g["nfree"])
    prop = q.propagator_cn_hc_lgwz().initialize(int(g["n_r"]), int(g["p"]), n_l, g["S"], g["R"], g["H"], dt)
    prop.put(g["init"][None])
    ts = _tsurff(q, g)
    prop.run_ex(g["field"][None, :nt + 1], [nt], [nt + nfree], tsurff=ts)
    work, clock = ts.get()
    assert rel_l2(prop.get()[0], g["coef"]) < 1e-11
    assert np.abs(clock[0] - g["clock"]).max() < 1e-14
    assert rel_l2(work[0], g["work"]) < 1e-10


def test_tsurff_and_mask_run_uneven_batch(q):
    """t-SURFF then mask after every step, three instances with their own pulses and step
    counts: the device loop against the host loop of propagate + accumulate + mask"""
    g, m = golden("tsurff_small"), golden("small_mask")
    s = golden("small_setup")
    assert int(g["n_r"]) == int(s["n_r"]) and int(g["n_l"]) == int(s["n_l"])
    n_r, p, n_l, dt = int(g["n_r"]), int(g["p"]), int(g["n_l"]), float(g["dt"])
    B = 3
    c0 = np.stack([g["init"] * np.exp(0.2j * k) for k in range(B)])
    f = g["field"]
    nt = int(g["nt"])
    ftab = np.stack([f[:nt + 1] * (1.0 + 0.2 * k) for k in range(B)])
    nf = np.array([nt, nt // 2, 0])
    ntt = np.array([nt + 4, nt - 3, 6])
    run = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, g["S"], g["R"], g["H"], dt, n_inst=B)
    run.put(c0)
    ts = _tsurff(q, g, B)
    run.run_ex(ftab, nf, ntt, mask=m["band"], tsurff=ts)
    work, clock = ts.get()
    out = run.get()
    for k in range(B):
        one = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, g["S"], g["R"], g["H"], dt)
        one.put(c0[k:k + 1])
        t1 = _tsurff(q, g)
        for i in range(ntt[k]):
            if i < nf[k]:
                one.propagate(ftab[k, i], ftab[k, i + 1])
                t1.accumulate(one, dt, (ftab[k, i], ftab[k, i + 1]))
            else:
                one.propagate()
                t1.accumulate(one, dt)
            one.mask(m["band"])
        w1, c1 = t1.get()
        assert rel_l2(out[k], one.get()[0]) < 1e-12, k
        assert np.abs(clock[k] - c1[0]).max() < 1e-14, k
        assert rel_l2(work[k], w1[0]) < 1e-12, k
        one.close()
        t1.close()
