"""The harmonic spectra of many dipole lists on the GPU (qpc_hhg_spectra) against the host
function (qpc_hhg_spectrum, analysis/plot_hhs.m restated and pinned to numpy's FFT in
tests/test_spectra.py): random lists of several lengths in one uneven batch, the reference's own
mid-pulse dipole list, both dipole types, and fewer frequencies than the full half spectrum."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dipole_type", [1, 2])
def test_batch_matches_host(q, dipole_type):
    rng = np.random.default_rng(5)
    ns = np.array([1, 2, 7, 64, 1000, 2407, 8826])
    ld = int(ns.max())
    z = np.zeros((ns.size, ld))
    for i, n in enumerate(ns):
        z[i, :n] = rng.standard_normal(n)
    dt, t0 = 0.05, 0.3
    tmin = t0 + 2 * dt * np.ones(ns.size)
    tmax = t0 + dt * np.maximum(ns - 3, 3)
    kmax = (ld + 1) // 2
    s = q.hhg_spectra(z, ns, dt, kmax, t0=t0, tmin=tmin, tmax=tmax, dipole_type=dipole_type)
    for i, n in enumerate(ns):
        _, sr = q.hhg_spectrum(z[i, :n], dt, t0, tmin[i], tmax[i], dipole_type)
        nh = (n + 1) // 2
        assert np.abs(s[i, :nh] - sr).max() <= 1e-12 * max(np.abs(sr).max(), 1e-300), n
        assert np.all(s[i, nh:] == 0.0)


def test_reference_dipole_and_partial_band(q):
    """the reference's z list (mid-pulse fixture): the first 300 frequencies equal the host
    spectrum's"""
    m = golden("mid_pulse")
    z = m["zlist"]
    dt = float(m["dt"])
    _, sr = q.hhg_spectrum(z, dt, 0.0, 0.0, dt * (z.size - 1))
    s = q.hhg_spectra(z[None], [z.size], dt, 300)
    assert np.all(np.isfinite(s)) and np.all(s >= 0)
    assert np.abs(s[0] - sr[:300]).max() <= 1e-12 * sr.max()
