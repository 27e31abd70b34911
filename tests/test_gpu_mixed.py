"""Mixed-grid batch: wavefunctions with their own radial grid, l_max and potential
V = -(1 + a e^{-b r})/r, advanced together -- the Crank-Nicolson propagator on one
handle per grid through qpc_lgwz_run_many, each instance against the CPU oracle
of the same propagator (1e-10 relative L2, one instance over its full pulse, the others
over 200 steps around their pulse peak, up to the largest grid of the mixed-grid batch:
N_r = 2000, l_max = 80)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

DT = 0.05


def pulse(q, rng, nc=None, lam=None):
    """A field drawn like the batched laser scan: I log-uniform in [5e13, 5e14] W/cm^2,
    wavelength uniform in [400, 2000] nm, CEP uniform in [0, 2 pi), cycles 2..10."""
    inten = 10 ** rng.uniform(np.log10(5e13), np.log10(5e14))
    lam = rng.uniform(400, 2000) if lam is None else lam
    cep = rng.uniform(0, 2)
    nc = int(rng.integers(2, 11)) if nc is None else nc
    return q.field_sinen(q.intensity_to_e0(inten), q.wavelength_to_w0(lam), nc, 0.0, cep, DT)


def instance(q, rng, n_r, n_l, p=6):
    a, b = rng.uniform(0, 17), rng.uniform(1, 3)
    S, R, _, _, H = q.radial_setup(n_r, p, n_l, q.linear_knots(n_r, p, 0.0, n_r / 2.0), (q.POTENTIAL_YUKAWA, 1.0, a, b))
    c0, _ = q.ground_state(S, H, n_l)
    return S, R, H, c0


def test_mixed_grid_cn_batch(q, oracle):
    rng = np.random.default_rng(2025)
    grids = [(400, 21), (800, 41), (1200, 21), (400, 61), (1600, 61), (2000, 81)]
    props, tabs, nts, cases = [], [], [], []
    for k, (n_r, n_l) in enumerate(grids):
        S, R, H, c0 = instance(q, rng, n_r, n_l)
        if k == 0:
            f = pulse(q, rng, nc=2, lam=400.0)      # the shortest pulse of the scan, in full
            nt = f.size - 1
        else:
            f = pulse(q, rng)
            mid = f.size // 2                     # 200 steps around the pulse peak
            f = f[mid - 100: mid + 101]
            nt = 200
        pr = q.propagator_cn_hc_lgwz().initialize(n_r, 6, n_l, S, R, H, DT)
        pr.put(c0[None])
        props.append(pr)
        tabs.append(f[None, :])
        nts.append(nt)
        cases.append((S, R, H, c0, f, nt, n_l))
    q.run_many(props, tabs, nts)
    for pr, (S, R, H, c0, f, nt, n_l) in zip(props, cases):
        g = oracle.grid(S, R, H, DT, n_l)
        ref = oracle.run(g, c0.reshape(1, -1), f[None, :], [nt], [nt], threads=4)
        assert rel_l2(pr.get().reshape(-1), ref[0]) < 1e-10, (S.shape[0], n_l)
        assert abs(pr.norm()[0] - oracle.norm(g, ref)[0]) < 1e-10


def test_run_many_reports_the_failing_handle(q):
    rng = np.random.default_rng(5)
    props = []
    for n_r, n_l in [(400, 21), (400, 21)]:
        S, R, H, c0 = instance(q, rng, n_r, n_l)
        pr = q.propagator_cn_hc_lgwz().initialize(n_r, 6, n_l, S, R, H, DT)
        pr.put(c0[None])
        props.append(pr)
    f = np.zeros((1, 11))
    f_bad = f.copy()
    f_bad[0, 3] = np.nan
    with pytest.raises(q.QpcError, match="handle 1"):
        q.run_many(props, [f, f_bad], [10, 10])


def test_own_potentials_in_one_handle(q, oracle):
    """five wavefunctions on one grid, each with its own screened potential and pulse (uneven step
    counts), in one handle (qpc_lgwz_create_ex): each against the oracle with its own Hamiltonian;
    the single-step path (propagate) against a run of the same steps"""
    rng = np.random.default_rng(77)
    n_r, n_l, B = 400, 21, 5
    insts = [instance(q, rng, n_r, n_l) for _ in range(B)]
    S, R = insts[0][0], insts[0][1]
    H = np.stack([x[2] for x in insts])
    c0 = np.stack([x[3] for x in insts])
    tabs, nts = [], []
    for k in range(B):
        f = pulse(q, rng, nc=2, lam=400.0 + 40.0 * k)
        tabs.append(f)
        nts.append(min(f.size - 1, 300 + 37 * k))
    ld = max(t.size for t in tabs)
    ftab = np.zeros((B, ld))
    for k, t in enumerate(tabs):
        ftab[k, :t.size] = t
    pr = q.propagator_cn_hc_lgwz().initialize(n_r, 6, n_l, S, R, H, DT, n_inst=B)
    pr.put(c0)
    pr.run(ftab, nts, [n + 20 for n in nts])
    out = pr.get()
    for k in range(B):
        g = oracle.grid(S, R, H[k], DT, n_l)
        ref = oracle.run(g, c0[k].reshape(1, -1), ftab[k:k + 1], [nts[k]], [nts[k] + 20], threads=4)
        assert rel_l2(out[k].reshape(-1), ref[0]) < 1e-10, k
    # one step through propagate() uses each instance's own factors too
    pr.put(c0)
    pr.propagate(ftab[:, 0], ftab[:, 1])
    one = pr.get()
    for k in range(B):
        g = oracle.grid(S, R, H[k], DT, n_l)
        ref = oracle.step(g, c0[k].reshape(1, -1), ftab[k, 0], ftab[k, 1])
        assert rel_l2(one[k].reshape(-1), ref[0]) < 1e-12, k
