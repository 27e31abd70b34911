"""Parity of the GB300 engine (through the C ABI) against the CPU oracle and
the reference's golden vectors.  Tolerance: relative L2 of the coefficients
<= 1e-10 after full pulses (the bar the path is held to); single steps and
short runs are held to 1e-12."""
import numpy as np
import pytest

from conftest import engine, golden, rel_l2

pytestmark = pytest.mark.gpu

TOL_FULL = 1e-10
TOL_SHORT = 1e-12


def grid(q, n_r, p, n_l, rmax, pot=None, n_lh=None):
    t = q.linear_knots(n_r, p, 0.0, rmax)
    args = (n_r, p, n_lh or n_l, t) + ((pot,) if pot else ())
    S, R, Ri, D, H = q.radial_setup(*args)
    return S, R, H


def rand_state(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.fixture(scope="module")
def small(q):
    g = golden("small_setup")
    return g


def test_single_step_matches_oracle(q, oracle, small):
    g = small
    n_r, p, n_l, dt = int(g["n_r"]), int(g["p"]), int(g["n_l"]), float(g["dt"])
    S, R, H = grid(q, n_r, p, n_l, float(g["rmax"]))
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt)
    c0 = rand_state(np.random.default_rng(3), 1, 1, n_l, n_r)
    prop.put(c0)
    prop.propagate(0.03, 0.045)
    og = oracle.grid(S, R, H, dt, n_l)
    ref = oracle.step(og, c0, 0.03, 0.045)
    assert rel_l2(prop.get(), ref.reshape(1, 1, n_l, n_r)) < TOL_SHORT
    prop.propagate()  # field-free overload
    ref = oracle.step(og, ref)
    assert rel_l2(prop.get(), ref.reshape(1, 1, n_l, n_r)) < TOL_SHORT


def test_golden_small_propagation(q, small):
    """Against the reference itself: 50 field steps + 5 field-free (tests/golden/small_prop)."""
    g = small
    pr = golden("small_prop")
    n_r, p, n_l, dt = int(g["n_r"]), int(g["p"]), int(g["n_l"]), float(g["dt"])
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, g["S"], g["R"], g["H"], dt)
    prop.put(pr["init"][None, None])
    nt, nf = int(pr["nt"]), int(pr["nfree"])
    prop.run(pr["f"][None, :], [nt], [nt + nf])
    c = prop.get()[0, 0]
    assert rel_l2(c, pr["coef"]) < TOL_SHORT
    assert abs(prop.norm()[0] - pr["norm"][0]) < 1e-12 * pr["norm"][0]
    z = prop.dipole(g["R"])[0]
    assert abs(z.real - pr["dipole"][0]) < 1e-11 * abs(pr["dipole"][0])


def test_stepwise_equals_run(q, small):
    """propagate() called step by step and run() over the same table agree."""
    g = small
    pr = golden("small_prop")
    n_r, p, n_l, dt = int(g["n_r"]), int(g["p"]), int(g["n_l"]), float(g["dt"])
    a = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, g["S"], g["R"], g["H"], dt)
    b = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, g["S"], g["R"], g["H"], dt)
    a.put(pr["init"][None, None])
    b.put(pr["init"][None, None])
    f = pr["f"]
    for i in range(20):
        a.propagate(f[i], f[i + 1])
    b.run(f[None, :21], [20])
    assert rel_l2(a.get(), b.get()) < TOL_SHORT


def test_uneven_batch_matches_oracle(q, oracle):
    """A batch whose instances carry their own fields and step counts (with
    field-free tails), against the oracle instance by instance."""
    n_r, p, n_l, dt = 96, 6, 9, 0.05
    S, R, H = grid(q, n_r, p, n_l, 48.0)
    B = 7
    rng = np.random.default_rng(11)
    nt_field = np.array([0, 1, 2, 37, 60, 15, 60])
    nt_total = nt_field + np.array([3, 0, 5, 1, 0, 20, 7])
    ld = nt_field.max() + 1
    ftab = np.zeros((B, ld))
    for k in range(B):
        ftab[k, :nt_field[k] + 1] = rng.uniform(0.02, 0.1) * np.sin(rng.uniform(0.05, 0.2) * np.arange(nt_field[k] + 1) + rng.uniform(0, 6))
    c0 = rand_state(rng, B, 1, n_l, n_r)
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt, n_inst=B)
    prop.put(c0)
    prop.run(ftab, nt_field, nt_total)
    got = prop.get()
    og = oracle.grid(S, R, H, dt, n_l, n_inst=B)
    ref = oracle.run(og, c0, ftab, nt_field, nt_total, threads=4)
    for k in range(B):
        assert rel_l2(got[k], ref[k]) < TOL_SHORT, k
    on = oracle.norm(og, ref)
    assert np.abs(prop.norm() - on).max() < 1e-12 * on.max()


@pytest.mark.parametrize("n_l,p,n_m,m0", [(8, 6, 1, 0), (7, 7, 1, 0), (6, 5, 3, -1), (5, 4, 2, 1)])
def test_other_grids_match_oracle(q, oracle, n_l, p, n_m, m0):
    """Even n_l (no zero eigenvalue), other B-spline degrees, several m."""
    n_r, dt = 72, 0.04
    lmax = max(abs(m0), abs(m0 + n_m - 1)) + n_l - 1
    S, R, H = grid(q, n_r, p, n_l, 40.0, n_lh=lmax + 1)
    rng = np.random.default_rng(5 + n_l)
    c0 = rand_state(rng, 2, n_m, n_l, n_r)
    nt = 12
    ftab = 0.06 * np.sin(0.3 * np.arange(nt + 1))[None, :].repeat(2, 0)
    ftab[1] *= -0.7
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt, n_m=n_m, m0=m0, n_inst=2)
    prop.put(c0)
    prop.run(ftab, [nt, nt], [nt, nt + 2])
    og = oracle.grid(S, R, H, dt, n_l, n_m=n_m, m0=m0, n_inst=2)
    ref = oracle.run(og, c0, ftab, [nt, nt], [nt, nt + 2], threads=2)
    assert rel_l2(prop.get(), ref) < TOL_SHORT


def test_golden_mid_pulse(q):
    """Reference output: ground state through one 800 nm cycle at 2e14 W/cm^2, then
    200 field-free steps, with the driver's per-step <z> (z_list)."""
    m = golden("mid_pulse")
    n_r, p, n_l, dt = int(m["n_r"]), int(m["p"]), int(m["n_l"]), float(m["dt"])
    S, R, H = grid(q, n_r, p, n_l, float(m["rmax"]))
    c0, _ = q.ground_state(S, H, n_l)
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt)
    prop.put(c0[None])
    nt, nf = int(m["nt"]), int(m["nfree"])
    z = prop.run_dipole(m["f"][None, :], [nt], [nt + nf], R)[0]
    c = prop.get()[0, 0]
    ref = m["coef"]
    sgn = np.sign(np.vdot(ref.ravel(), c.ravel()).real)
    assert rel_l2(sgn * c, ref) < TOL_FULL
    assert abs(prop.norm()[0] - m["norm"][0]) < 1e-10
    # <z>(t_i) at every step; the dipole is even in the state's sign
    zr = m["zlist"]
    assert z.shape == zr.shape
    assert np.abs(z - zr).max() < 1e-10 * np.abs(zr).max()


def test_golden_small_dipole_list(q, small):
    """Per-step <z> of a random state through 50 field + 5 field-free steps, against the reference."""
    g = small
    pr = golden("small_prop")
    n_r, p, n_l, dt = int(g["n_r"]), int(g["p"]), int(g["n_l"]), float(g["dt"])
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, g["S"], g["R"], g["H"], dt, n_inst=2)
    prop.put(np.repeat(pr["init"][None, None], 2, 0))
    nt, nf = int(pr["nt"]), int(pr["nfree"])
    z = prop.run_dipole(np.repeat(pr["f"][None, :], 2, 0), [nt, nt], [nt + nf, nt + nf], g["R"])
    zr = pr["zlist"]
    for k in range(2):
        assert np.abs(z[k] - zr).max() < 1e-11 * np.abs(zr).max()
    assert rel_l2(prop.get()[0, 0], pr["coef"]) < TOL_SHORT


def test_dipole_list_uneven_batch(q, oracle):
    """In-loop dipole for instances with their own pulses and field-free tails
    (the eigen-basis observation inside the coupling solve and the l-basis one
    after the pulse), against the oracle stepped one call at a time."""
    n_r, p, n_l, dt = 80, 6, 7, 0.05
    S, R, H = grid(q, n_r, p, n_l, 40.0)
    rng = np.random.default_rng(19)
    B = 4
    nt_field = np.array([0, 1, 9, 14])
    nt_total = nt_field + np.array([4, 3, 0, 2])
    ld = nt_field.max() + 1
    ftab = 0.05 * rng.standard_normal((B, ld))
    c0 = rand_state(rng, B, 1, n_l, n_r)
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt, n_inst=B)
    prop.put(c0)
    z = prop.run_dipole(ftab, nt_field, nt_total, R)
    og = oracle.grid(S, R, H, dt, n_l, n_inst=1)
    y10 = q.y10_coupling(n_l, 0)
    for k in range(B):
        c = c0[k:k + 1].copy()
        zr = []
        for s in range(nt_total[k]):
            zr.append(oracle.dipole(og, R, y10, c)[0].real)
            if s < nt_field[k]:
                c = oracle.step(og, c, ftab[k, s], ftab[k, s + 1])
            else:
                c = oracle.step(og, c)
        zr = np.array(zr)
        assert np.abs(z[k, :nt_total[k]] - zr).max() < 1e-11 * max(1.0, np.abs(zr).max()), k
        assert np.all(z[k, nt_total[k]:] == 0.0)
        assert rel_l2(prop.get()[k], c.reshape(1, n_l, n_r)) < TOL_SHORT


def test_golden_c0_full_pulse(q):
    """The C0 workload against the reference: 8826 steps, H atom, N_r=400, l_max=20."""
    g = golden("c0_final")
    fz = golden("c0_field")["f"]
    n_r, p, n_l, dt = int(g["n_r"]), int(g["p"]), int(g["n_l"]), float(g["dt"])
    S, R, H = grid(q, n_r, p, n_l, float(g["rmax"]))
    c0, e = q.ground_state(S, H, n_l)
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt)
    prop.put(c0[None])
    nt = fz.size - 1
    prop.run(fz[None, :], [nt])
    c = prop.get()[0, 0]
    ref = g["coef"]
    sgn = np.sign(np.vdot(ref.ravel(), c.ravel()).real)
    err = rel_l2(sgn * c, ref)
    drift = abs(prop.norm()[0] - 1.0)
    print("C0 rel L2 vs reference %.3e, |1-norm| %.3e (reference %.3e)" % (err, drift, abs(g["norm"][0] - 1)))
    assert err < TOL_FULL
    assert drift < 1e-10
    # dipole and projections (PES) at the end of the pulse
    z = prop.dipole(R)[0]
    assert abs(z.real - g["dipole"][0]) < 1e-9 * max(1.0, abs(g["dipole"][0]))
    nnz = g["proj_nnz"]
    basis, off = [], 0
    for l in range(n_l):
        e_l, v_l = q.gen_eigen(S, H[l], int(nnz[l]))
        # left vectors S v, as eigenstate_sph stores them
        Sv = np.zeros_like(v_l)
        for j in range(v_l.shape[0]):
            x = v_l[j]
            y = np.zeros(n_r)
            for r in range(n_r):
                for k in range(p + 1):
                    if r + k < n_r:
                        y[r] += S[r, k] * x[r + k]
                        if k:
                            y[r + k] += S[r, k] * x[r]
            Sv[j] = y
        basis.append(Sv)
    proj = prop.projection(nnz.astype(np.int32), basis)
    # the reference keeps proj[m][l][0:n_r] with the first proj_nnz[l] entries used
    ref = np.concatenate([g["proj"][il * n_r: il * n_r + int(nnz[il])] for il in range(n_l)])
    assert proj.shape == ref.shape
    # eigenvector signs are arbitrary: compare |<v|c>|^2 (what the spectrum uses)
    assert np.abs(np.abs(proj) ** 2 - np.abs(ref) ** 2).max() < 1e-10


def test_deterministic(q, small):
    g = small
    pr = golden("small_prop")
    n_r, p, n_l, dt = int(g["n_r"]), int(g["p"]), int(g["n_l"]), float(g["dt"])
    outs = []
    for _ in range(2):
        prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, g["S"], g["R"], g["H"], dt, n_inst=3)
        prop.put(np.repeat(pr["init"][None, None], 3, 0))
        prop.run(np.repeat(pr["f"][None, :], 3, 0), [50, 20, 35])
        outs.append((prop.get(), prop.norm()))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])


def test_field_free_stationary_phase(q):
    """A field-free eigenstate only picks up the CN phase exactly:
    c(n dt) = ((1 - i E dt/2)/(1 + i E dt/2))^n c(0)."""
    n_r, p, n_l, dt = 80, 6, 4, 0.05
    S, R, H = grid(q, n_r, p, n_l, 40.0)
    c0, e = q.ground_state(S, H, n_l)
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt)
    prop.put(c0[None])
    n = 500
    prop.run(None, [0], [n])
    ph = ((1 - 0.5j * e * dt) / (1 + 0.5j * e * dt)) ** n
    assert rel_l2(prop.get()[0, 0], ph * c0) < 1e-11


def test_zero_pivot_is_reported_not_trapped(q):
    """A singular band (S = 0) is an error code from create, no device fault."""
    n_r, p, n_l = 32, 6, 3
    S = np.zeros((n_r, p + 1))
    H = np.zeros((n_l, n_r, p + 1))
    with pytest.raises(q.QpcError) as e:
        q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, S, H, 0.05)
    assert e.value.code == 4


def test_mask_matches_reference(q):
    """absorber_mask applied by the engine to its resident state (tests/golden/small_mask)."""
    s, m = golden("small_setup"), golden("small_mask")
    n_r, p, n_l = int(s["n_r"]), int(s["p"]), int(s["n_l"])
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, s["S"], s["R"], s["H"], float(s["dt"]), n_inst=2)
    prop.put(np.stack([m["init"], 2.0 * m["init"]])[:, None])
    prop.mask(m["band"])
    out = prop.get()
    assert rel_l2(out[0, 0], m["coef"]) < 1e-13
    assert rel_l2(out[1, 0], 2.0 * m["coef"]) < 1e-13


def test_masked_driver_loop_matches_oracle(q, oracle, aoracle):
    """The reference driver's propagate-then-mask loop (sphTDSE.cpp:799-810) for 20 steps."""
    s, m = golden("small_setup"), golden("small_mask")
    n_r, p, n_l, dt = int(s["n_r"]), int(s["p"]), int(s["n_l"]), float(s["dt"])
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, s["S"], s["R"], s["H"], dt)
    og = oracle.grid(s["S"], s["R"], s["H"], dt, n_l)
    chol = golden("arnoldi_small")["chol"]
    c = m["init"].reshape(1, -1).copy()
    prop.put(c.reshape(1, 1, n_l, n_r))
    f = 0.05 * np.sin(0.1 * np.arange(21))
    for i in range(20):
        prop.propagate(f[i], f[i + 1])
        prop.mask(m["band"])
        c = oracle.step(og, c, f[i], f[i + 1])
        c = aoracle.mask(m["band"], chol, c.reshape(-1), n_l).reshape(1, -1)
    assert rel_l2(prop.get().reshape(-1), c[0]) < 1e-12


def test_golden_multi_m(q):
    """Several m (m = -2..2) against the reference's own propagator (tests/golden/ep_prop)."""
    g = golden("ep_prop")
    n_r, p, n_l, n_m, m0 = int(g["n_r"]), int(g["p"]), int(g["n_l"]), int(g["n_m"]), int(g["m0"])
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, g["S"], g["R"], g["H"], float(g["dt"]), n_m=n_m, m0=m0)
    prop.put(g["init"][None])
    nt, nf = int(g["nt"]), int(g["nfree"])
    prop.run(g["f"][None, :], [nt], [nt + nf])
    assert rel_l2(prop.get()[0], g["coef"]) < 1e-12
    assert abs(prop.norm()[0] - g["norm"][0]) < 1e-12 * g["norm"][0]


def test_full_size_batched_scan_window(q, oracle):
    """The 256-wavefunction scan at its full size (N_r = 800 on [0, 400], p = 6, l < 41, fields drawn as
    the benchmark draws them): 200 steps of the whole batch, three instances against the oracle, and
    the S-norm of every instance conserved (the Crank-Nicolson step is S-unitary)."""
    n_r, p, n_l, dt, B, K = 800, 6, 41, 0.05, 256, 200
    S, R, H = grid(q, n_r, p, n_l, 400.0)
    c0, _ = q.ground_state(S, H, n_l)
    rng = np.random.default_rng(2025)
    inten = 10 ** rng.uniform(np.log10(5e13), np.log10(5e14), B)
    lam = rng.uniform(400.0, 2000.0, B)
    cep = rng.uniform(0.0, 2 * np.pi, B)
    cyc = rng.integers(2, 11, B)
    ftab = np.stack([q.field_sinen(q.intensity_to_e0(I), q.wavelength_to_w0(l), float(c), 0.0, float(ph / np.pi), dt)[:K + 1]
                     for I, l, ph, c in zip(inten, lam, cep, cyc)])
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt, n_inst=B)
    state = np.repeat(c0[None], B, 0)
    prop.put(state)
    n0 = prop.norm()
    prop.run(ftab, np.full(B, K))
    out = prop.get()
    assert np.abs(prop.norm() - n0).max() < 1e-11 * n0.max()
    g = oracle.grid(S, R, H, dt, n_l)
    for k in (0, 97, 255):
        ref = oracle.run(g, c0.reshape(1, -1), ftab[k:k + 1], [K], [K], threads=4)
        assert rel_l2(out[k].reshape(-1), ref[0]) < 1e-11, k   # 200 steps of the large grid: 1.4e-12 measured
