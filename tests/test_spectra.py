"""Spectra post-processing (host): the harmonic spectrum of analysis/plot_hhs.m,
the photoelectron energy spectrum and the ionization yield."""
import numpy as np
import pytest

from conftest import golden


def _hhg_reference(z, dt, t0, tmin, tmax, dipole_type):
    # analysis/plot_hhs.m written out with numpy's FFT
    n = z.size
    t = t0 + dt * np.arange(n)
    win = ((t > tmin) & (t < tmax)) * np.sin(np.pi * (t - tmin) / (tmax - tmin)) ** 2
    d = np.fft.fft(-z * win) * dt / (2 * np.pi)
    nh = (n + 1) // 2
    w = np.arange(nh) * 2 * np.pi / (dt * n)
    with np.errstate(divide="ignore"):
        fac = w ** 2 if dipole_type == 1 else np.where(w > 0, 1.0 / np.where(w > 0, w, 1.0) ** 2, 0.0)
    return w, 4 * np.pi ** 2 * fac / 137.036 ** 2 * np.abs(d[:nh]) ** 2


@pytest.mark.parametrize("n", [1, 2, 7, 64, 1000, 2407, 8826])
@pytest.mark.parametrize("dipole_type", [1, 2])
def test_hhg_matches_plot_hhs(q, n, dipole_type):
    rng = np.random.default_rng(n)
    z = rng.standard_normal(n)
    dt, t0 = 0.05, 0.3
    tmin, tmax = t0 + 2 * dt, t0 + dt * max(n - 3, 3)
    w, s = q.hhg_spectrum(z, dt, t0, tmin, tmax, dipole_type)
    wr, sr = _hhg_reference(z, dt, t0, tmin, tmax, dipole_type)
    assert np.abs(w - wr).max() < 1e-12
    assert np.abs(s - sr).max() <= 1e-13 * max(np.abs(sr).max(), 1e-300)


def test_hhg_of_the_reference_dipole(q):
    """Spectrum of the reference's own z_list (mid-pulse fixture) through the engine's
    function equals plot_hhs.m written with numpy's FFT; non-negative and finite."""
    m = golden("mid_pulse")
    z = m["zlist"]
    dt = float(m["dt"])
    w, s = q.hhg_spectrum(z, dt, 0.0, 0.0, dt * (z.size - 1))
    wr, sr = _hhg_reference(z, dt, 0.0, 0.0, dt * (z.size - 1), 1)
    assert np.all(np.isfinite(s)) and np.all(s >= 0)
    assert np.abs(s - sr).max() <= 1e-12 * sr.max()


def test_pes_and_yield(q):
    rng = np.random.default_rng(3)
    pr = rng.standard_normal(200) + 1j * rng.standard_normal(200)
    en = rng.uniform(-1.0, 3.0, 200)
    pes, bound, yld = q.pes_bin(pr, en, 0.0, 2.0, 16)
    w = np.abs(pr) ** 2
    assert abs(bound - w[en < 0].sum()) < 1e-12 * w.sum()
    assert abs(yld - (1.0 - bound)) < 1e-15
    edges = np.linspace(0.0, 2.0, 17)
    ref, _ = np.histogram(en, bins=edges, weights=w)
    assert np.abs(pes * (2.0 / 16) - ref).max() < 1e-12 * w.sum()


def test_yield_from_reference_projections(q):
    """Ionization yield of the C0 run from the reference's own projections: the bound
    population is the |proj|^2 of states with E < 0, per (m, l) channel."""
    g = golden("c0_final")
    n_r = int(g["n_r"])
    nnz = g["proj_nnz"]
    pr = np.concatenate([g["proj"][il * n_r: il * n_r + int(nnz[il])] for il in range(int(g["n_l"]))])
    en = g["proj_energy"]
    pes, bound, yld = q.pes_bin(pr, en, 0.0, 2.0, 64)
    assert 0.0 < yld < 0.2 and 0.8 < bound < 1.0
    assert abs(bound + pes.sum() * (2.0 / 64) - (np.abs(pr) ** 2).sum()) < 1e-12
