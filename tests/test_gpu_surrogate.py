"""The spectra surrogate end to end on a small grid: TDSE labels from the batched
engine, GPU training of the ensemble, and the trust gate that routes queries to the
TDSE fallback (fallback answers equal the TDSE labels; ellipticity != 0 is refused
by the z-linear engine)."""
import importlib
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRID = dict(n_r=200, p=6, n_l=11, rmax=100.0, dt=0.05)


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
    # elliptical queries are out of trust and need an elliptical propagator
    q6["ellipticity"] = np.full(6, 0.5)
    with pytest.raises(ValueError):
        s.query(q6, threshold=np.inf, setup=setup)
