"""Parity of the GPU Arnoldi propagator (propagator_hc_lgwz of la_1e.hpp, through the
C ABI) against the reference's golden vectors and the CPU oracle.

Tolerances: single steps and short runs 1e-12 relative L2; full runs 1e-10 where
the Krylov step is well conditioned.  At kmax = 12, dt = 0.1 on grids with
spacing 0.5 a.u. the reference's own map is not: a 1e-15 change of its input moves
its result by up to percent over a pulse (Krylov vectors formed by cancellation
when <v|S|v> is small, and components outside the Krylov space multiplied by the
interpolating polynomial).  There the GPU is held per step to the oracle applied
to the GPU's own input (1e-11).  Run-level checks take well-conditioned cases and
allow 100 x the oracle's own spread under a 1e-15 perturbation of the input only
while that spread is itself tiny (the bound fails the test otherwise)."""
import numpy as np
import pytest

from conftest import engine, golden, rel_l2

pytestmark = pytest.mark.gpu

TOL_SHORT = 1e-12
TOL_FULL = 1e-10


def small_prop(q, n_inst=1, H=None, dt=0.1, kmax=12):
    s = golden("small_setup")
    return q.propagator_hc_lgwz(kmax, 1e-14, 1e-8).initialize(
        int(s["n_r"]), int(s["p"]), int(s["n_l"]), s["S"], s["R"], s["H"] if H is None else H, s["y10"], dt,
        n_inst=n_inst)


def oracle_with_spread(aoracle, g, c0, ez, nt=None):
    """The oracle's result, criterion codes and Krylov dimensions, and per instance the
    tolerance max(TOL_SHORT, 100 x the largest change of its result under two 1e-15
    relative perturbations of the input).  The factor covers that two implementations
    differ by rounding in every step, not only in the input.  Codes are compared only
    where the perturbed runs keep them."""
    ref, crit, ms = aoracle.run(g, c0, ez, nt)
    tol = np.full(ref.shape[0], TOL_SHORT)
    stable = np.ones(crit.shape, bool)
    for seed in (99, 100):
        noise = 1 + 1e-15 * np.random.default_rng(seed).standard_normal(c0.shape)
        ref2, crit2, ms2 = aoracle.run(g, c0 * noise, ez, nt)
        tol = np.maximum(tol, [100 * rel_l2(ref2[k], ref[k]) for k in range(ref.shape[0])])
        stable &= (crit == crit2) & (ms == ms2)
    # a spread this large means the reference's map is ill-conditioned on this case and the
    # bound would accept a wrong answer: such a case cannot be checked at run level
    assert tol.max() <= 1e-10, "oracle spread too large for a run-level check: %s" % tol
    return ref, crit, ms, tol, stable


def test_golden_converged_run(q):
    """3000 steps of dt = 0.01 against the reference (criterion 2 throughout)."""
    s, a = golden("small_setup"), golden("arnoldi_small")
    prop = small_prop(q, dt=float(a["conv_dt"]))
    prop.put(s["gs_coef"][None, None])
    crit = prop.run(a["conv_ez"][None, :])
    assert rel_l2(prop.get()[0, 0], a["conv_coef"]) < TOL_FULL
    assert np.array_equal(crit[0], a["conv_crit"])
    assert abs(prop.norm()[0] - 1.0) < 1e-12


def test_golden_steps_batch_per_instance_potential(q):
    """One batch, two Hamiltonians: instance 0 hydrogen, instance 1 Yukawa, both from
    the same state; against the reference's step1 and ystep1."""
    s, a = golden("small_setup"), golden("arnoldi_small")
    H = np.stack([s["H"], golden("small_yukawa")["H"]])
    prop = small_prop(q, n_inst=2, H=H, dt=float(a["step1_dt"]))
    prop.put(np.stack([a["conv_coef"], a["conv_coef"]])[:, None])
    crit = prop.propagate(0.05)
    c = prop.get()
    assert rel_l2(c[0, 0], a["step1_coef"]) < TOL_SHORT
    assert rel_l2(c[1, 0], a["ystep1_coef"]) < TOL_SHORT
    assert crit[0] == a["step1_crit"][0] and crit[1] == a["ystep1_crit"][0]


def test_golden_three_steps(q):
    a = golden("arnoldi_small")
    prop = small_prop(q, dt=float(a["step3_dt"]))
    prop.put(a["conv_coef"][None, None])
    crit = prop.run(a["step3_ez"][None, :])
    # three steps of dt = 0.1 already amplify rounding ~10x (see the module docstring)
    assert rel_l2(prop.get()[0, 0], a["step3_coef"]) < 1e-11
    assert np.array_equal(crit[0], a["step3_crit"])


def test_golden_breakdown(q):
    """Field-free steps of an eigenstate stop the expansion at m = 1."""
    s, a = golden("small_setup"), golden("arnoldi_small")
    prop = small_prop(q, dt=float(a["bd_dt"]))
    prop.put(s["gs_coef"][None, None])
    crit, ms = prop.run(a["bd_ez"][None, :], want_msub=True)
    assert rel_l2(prop.get()[0, 0], a["bd_coef"]) < 1e-13
    assert np.all(ms == 1) and np.array_equal(crit[0], a["bd_crit"])


@pytest.mark.parametrize("tag", ["step1", "step2"])
def test_golden_mid_steps(q, tag):
    m, a = golden("mid_pulse"), golden("arnoldi_mid")
    n_r, p, n_l, rmax = int(m["n_r"]), int(m["p"]), int(m["n_l"]), float(m["rmax"])
    S, R, _, _, H = q.radial_setup(n_r, p, n_l, q.linear_knots(n_r, p, 0.0, rmax))
    prop = q.propagator_hc_lgwz(int(a["kmax"]), 1e-14, 1e-8).initialize(n_r, p, n_l, S, R, H, q.y10_coupling(n_l),
                                                                        float(a[tag + "_dt"]))
    prop.put(a["init"][None, None])
    crit = prop.run(a[tag + "_ez"][None, :])
    assert rel_l2(prop.get()[0, 0], a[tag + "_coef"]) < 1e-11
    assert np.array_equal(crit[0], a[tag + "_crit"])


def test_uneven_batch_matches_oracle(q, aoracle):
    """Four instances, own field tables and step counts (one takes no step); dt = 0.01, where
    the reference's map is well conditioned on this grid."""
    s = golden("small_setup")
    a = golden("arnoldi_small")
    rng = np.random.default_rng(7)
    B, n_l, n_r = 4, int(s["n_l"]), int(s["n_r"])
    c0 = np.stack([a["conv_coef"] * np.exp(1j * k) for k in range(B)])
    ez = 0.06 * rng.standard_normal((B, 6))
    nt = np.array([6, 0, 3, 5])
    prop = small_prop(q, n_inst=B, dt=0.01)
    prop.put(c0[:, None])
    crit, ms = prop.run(ez, nt, want_msub=True)
    g = aoracle.grid(s["S"], s["R"], s["H"], s["y10"], 0.01, n_l, n_inst=B)
    ref, rcrit, rms, tol, stable = oracle_with_spread(aoracle, g, c0.reshape(B, -1), ez, nt)
    c = prop.get().reshape(B, -1)
    for k in range(B):
        assert rel_l2(c[k], ref[k]) < tol[k], (k, tol[k])
    assert np.array_equal(crit[stable], rcrit[stable]) and np.array_equal(ms[stable], rms[stable])
    assert np.array_equal(crit[1], np.full(6, -1)) and np.array_equal(crit[2, 3:], np.full(3, -1))
    assert np.array_equal(c[1], c0[1].reshape(-1))


def test_several_m_matches_oracle(q, aoracle):
    """n_m = 3, m = -1, 0, 1: per-m couplings y10(m, l) and H_{|m|+il}."""
    n_r, p, n_l, n_m, m0 = 48, 5, 5, 3, -1
    lmax = 1 + n_l - 1
    S, R, _, _, H = q.radial_setup(n_r, p, lmax + 1, q.linear_knots(n_r, p, 0.0, 24.0))
    y10 = np.stack([q.y10_coupling(n_l, m0 + im) for im in range(n_m)])
    rng = np.random.default_rng(11)
    c0 = np.zeros((n_m, n_l, n_r), complex)
    for im in range(n_m):
        c0[im, 0] = q.ground_state(S, H, n_l, n_m, im, 0, 0, m0)[0][im, 0]
    c0[:, 1] += 0.1 * (rng.standard_normal((n_m, n_r)) * np.exp(-np.arange(n_r) / 8.0))
    prop = q.propagator_hc_lgwz(12, 1e-14, 1e-8).initialize(n_r, p, n_l, S, R, H, y10, 0.01, n_m=n_m, m0=m0)
    prop.put(c0[None])
    ez = 0.04 * np.sin(0.3 * np.arange(8))
    crit = prop.run(ez[None, :])
    g = aoracle.grid(S, R, H, y10, 0.01, n_l, n_m=n_m, m0=m0)
    ref, rcrit, _, tol, stable = oracle_with_spread(aoracle, g, c0.reshape(1, -1), ez)
    assert rel_l2(prop.get().reshape(-1), ref[0]) < tol[0]
    assert np.array_equal(crit[stable], rcrit[stable])
    # one step from the same input: within 1e-12
    prop.put(c0[None])
    prop.propagate(ez[1])
    ref1, _, _ = aoracle.run(g, c0.reshape(1, -1), ez[1:2])
    assert rel_l2(prop.get().reshape(-1), ref1[0]) < TOL_SHORT


def _mixed_instance(q, rng, n_r, n_l):
    """A mixed-grid workload instance: N_r B-splines on [0, N_r/2], l < n_l,
    V = -(1 + a e^{-b r})/r with a in [0, 17], b in [1, 3]."""
    a, b = rng.uniform(0, 17), rng.uniform(1, 3)
    p = 6
    pot = (q.POTENTIAL_YUKAWA, 1.0, a, b)
    S, R, _, _, H = q.radial_setup(n_r, p, n_l, q.linear_knots(n_r, p, 0.0, n_r / 2.0), pot)
    c0, e0 = q.ground_state(S, H, n_l)
    return S, R, H, c0, e0


@pytest.mark.parametrize("n_r,n_l", [(400, 21), (800, 41), (1600, 61), (2000, 81)])
def test_mixed_grid_shadowing(q, aoracle, n_r, n_l):
    """kmax = 12, dt = 0.1: every GPU step equals the oracle's step of the GPU's own
    input to 1e-11, along a trajectory through a field ramp."""
    rng = np.random.default_rng(n_r + n_l)
    S, R, H, c0, _ = _mixed_instance(q, rng, n_r, n_l)
    y10 = q.y10_coupling(n_l)
    prop = q.propagator_hc_lgwz(12, 1e-14, 1e-8).initialize(n_r, 6, n_l, S, R, H, y10, 0.1)
    g = aoracle.grid(S, R, H, y10, 0.1, n_l)
    prop.put(c0[None])
    ez = 0.05 * np.sin(0.057 * 0.1 * np.arange(12) + 0.4)
    worst = 0.0
    for s in range(ez.size):
        x = prop.get().reshape(1, -1)
        crit = prop.propagate(ez[s])
        ref, rcrit, _ = aoracle.run(g, x, ez[s:s + 1])
        worst = max(worst, rel_l2(prop.get().reshape(-1), ref[0]))
        assert crit[0] == rcrit[0, 0]
    assert worst < 1e-11
    assert abs(prop.norm()[0] - 1.0) < 1e-11


def test_mixed_grid_run_within_reference_spread(q, aoracle):
    """A 2000-step run at kmax = 12 on a screened-potential instance where the reference's map
    is well conditioned (64 splines on [0, 30], l < 6, dt = 0.01: criterion 2 throughout).  The
    GPU result differs from the oracle's by at most max(1e-10, 100 x the oracle's own change
    under a 1e-15 relative perturbation of the input), the spread itself must stay below
    1e-8 so that the bound cannot pass a wrong answer, and the S-norm is conserved.

    On the mixed-grid batch's grids (spacing 0.5 a.u., l_max >= 20, dt = 0.1) the reference's
    map is not continuous at that level: a 1e-15 perturbation moves its 400-step result by
    1e-3 to 1 (the early steps stop at the absolute 1e-13 breakdown threshold or not, and
    Gram-Schmidt on nearly cancelled vectors amplifies rounding).  There the GPU is held per
    step (test_mixed_grid_shadowing) instead."""
    rng = np.random.default_rng(3)
    n_r, n_l, dt = 64, 6, 0.01
    a, b = rng.uniform(0, 17), rng.uniform(1, 3)
    S, R, _, _, H = q.radial_setup(n_r, 6, n_l, q.linear_knots(n_r, 6, 0.0, 30.0), (q.POTENTIAL_YUKAWA, 1.0, a, b))
    c0, _ = q.ground_state(S, H, n_l)
    y10 = q.y10_coupling(n_l)
    nt = 2000
    t = dt * np.arange(nt)
    ez = 0.053 * np.sin(np.pi * t / (t[-1] + dt)) ** 2 * np.sin(0.0759 * t)
    g = aoracle.grid(S, R, H, y10, dt, n_l)
    ref, rcrit, _ = aoracle.run(g, c0.reshape(1, -1), ez)
    spread = 0.0
    for seed in (1, 2):
        pert = c0.reshape(1, -1) * (1 + 1e-15 * np.random.default_rng(seed).standard_normal(c0.size))
        ref2, _, _ = aoracle.run(g, pert, ez)
        spread = max(spread, rel_l2(ref2[0], ref[0]))
    assert spread < 1e-8, "the reference's map is ill-conditioned here (spread %.1e): no run-level check possible" % spread
    prop = q.propagator_hc_lgwz(12, 1e-14, 1e-8).initialize(n_r, 6, n_l, S, R, H, y10, dt)
    prop.put(c0[None])
    crit = prop.run(ez[None, :])
    err = rel_l2(prop.get().reshape(-1), ref[0])
    assert err <= max(TOL_FULL, 100 * spread), (err, spread)
    assert np.array_equal(crit[0], rcrit[0])
    assert abs(prop.norm()[0] - 1.0) < 1e-10


def test_deterministic(q):
    a = golden("arnoldi_small")
    out = []
    for _ in range(2):
        prop = small_prop(q, n_inst=3)
        prop.put(np.stack([a["conv_coef"]] * 3)[:, None])
        prop.run(np.array([[0.05, 0.02, -0.03]] * 3))
        out.append(prop.get())
    assert np.array_equal(out[0], out[1])
