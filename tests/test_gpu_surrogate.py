"""The spectra surrogate end to end on a small grid: TDSE labels from the batched
engine, GPU training of the ensemble, and the trust gate that routes queries to the
TDSE fallback (fallback answers equal the TDSE labels); queries with ellipticity != 0
are always answered by the velocity-gauge elliptical TDSE engine."""
import importlib
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRID = dict(n_r=200, p=6, n_l=11, rmax=100.0, dt=0.05)
ELL = dict(n_r=120, p=6, l_max=6, rmax=60.0, dt=0.05)


@pytest.fixture(scope="module")
def sg():
    return importlib.import_module("qpc-tdse-cpc_gb300.surrogate")


def small_params(sg, n, seed):
    p = sg.draw_params(n, seed)
    p["wavelength"] = np.random.default_rng(seed).uniform(400, 800, n)   # short pulses keep the test fast
    p["cycles"][:] = 2.0
    return p


def test_surrogate_pipeline(sg):
    p = small_params(sg, 48, 1)
    setup = sg._Setup(GRID, emax=max(3.17 * float(sg.up(p).max()) * 1.5, 1.0))
    t0 = time.perf_counter()
    pes, hhg, info = sg.tdse_spectra(p, grid=GRID, batch=24, setup=setup)
    tdse_s = time.perf_counter() - t0
    assert pes.shape == (48, sg.N_PES) and hhg.shape == (48, sg.N_HHG)
    assert np.all(np.isfinite(pes)) and np.all(np.isfinite(hhg))
    assert info["wf_steps"] > 0
    # labels do not depend on the batch they were computed in
    pes2, hhg2, _ = sg.tdse_spectra({k: v[:5] for k, v in p.items()}, grid=GRID, batch=5, setup=setup)
    assert np.allclose(pes2, pes[:5], atol=1e-9) and np.allclose(hhg2, hhg[:5], atol=1e-9)
    s = sg.Surrogate(n_members=5, n_hidden=64, n_layers=2, seed=3)
    hist = s.fit(p, pes, hhg, epochs=40, batch=16, lr=2e-3)
    assert np.all(hist[-1] < hist[0])
    mean, dis = s.predict(p)
    assert mean.shape == (48, sg.N_PES + sg.N_HHG) and np.all(dis >= 0)
    # what the network gains: the same 48 answers in a small fraction of the TDSE time
    t0 = time.perf_counter()
    s.predict(p)
    net_s = time.perf_counter() - t0
    assert net_s * 20 < tdse_s, (net_s, tdse_s)
    # trust everything: no fallback
    out, fall = s.query({k: v[:6] for k, v in p.items()}, threshold=np.inf, setup=setup)
    assert not fall.any()
    # trust nothing: every answer is the TDSE's
    q6 = {k: v[:6] for k, v in p.items()}
    out, fall = s.query(q6, threshold=-1.0, setup=setup)
    assert fall.all()
    ref = np.concatenate([pes[:6], hhg[:6]], axis=1)
    assert np.allclose(out, ref, atol=1e-9)
    # elliptical queries are out of trust whatever the ensemble says: the velocity-gauge TDSE answers
    q2 = {k: v[:2].copy() for k, v in p.items()}
    q2["ellipticity"] = np.array([0.5, -0.3])
    q2["wavelength"] = np.array([400.0, 450.0])
    ell_setup = sg._EllSetup(ELL, emax=max(3.17 * float(sg.up(q2).max()) * 1.5, 1.0))
    out, fall = s.query(q2, threshold=np.inf, setup=setup, ell_grid=ELL, ell_setup=ell_setup)
    assert fall.all()
    epes, ehhg, einfo = sg.tdse_spectra_elliptical(q2, grid=ELL, setup=ell_setup)
    assert einfo["wf_steps"] > 0 and np.all(np.isfinite(epes)) and np.all(np.isfinite(ehhg))
    assert np.allclose(out, np.concatenate([epes, ehhg], axis=1), atol=1e-9)
    # an ellipticity-0.5 pulse has a harmonic spectrum unlike the linear one of the same parameters
    lin = {k: v[:1].copy() for k, v in q2.items()}
    lin["ellipticity"] = np.zeros(1)
    lpes, lhhg, _ = sg.tdse_spectra_elliptical(lin, grid=ELL, setup=ell_setup)
    assert np.linalg.norm(lhhg[0] - ehhg[0]) > 1e-3 * np.linalg.norm(lhhg[0])


def test_elliptical_fallback_linear_pulse(sg):
    """At ellipticity 0 the velocity-gauge fallback sees a pulse along x: finite labels, the low
    harmonic orders decades above the high ones (the short pulse has no plateau up there)."""
    p = {"intensity": np.array([1e14]), "wavelength": np.array([400.0]), "cep": np.array([0.0]),
         "cycles": np.array([2.0]), "ellipticity": np.zeros(1)}
    ell_setup = sg._EllSetup(ELL, emax=max(3.17 * float(sg.up(p).max()) * 1.5, 1.0))
    pes, hhg, info = sg.tdse_spectra_elliptical(p, grid=ELL, setup=ell_setup)
    assert info["wf_steps"] > 0
    assert np.all(np.isfinite(pes)) and np.all(np.isfinite(hhg))
    assert hhg[0, :8].max() > hhg[0, -32:].max() + 2.0
