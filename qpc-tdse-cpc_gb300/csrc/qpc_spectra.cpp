// Spectra from the engine's outputs: harmonic spectrum from the per-step dipole,
// photoelectron energy spectrum and ionization yield from the projections onto
// field-free eigenstates.  Host-side post-processing, once per wavefunction.
#include "qpc_internal.h"
#include <cmath>
#include <complex>
#include <vector>

namespace qpc {

using cd = std::complex<double>;

// iterative radix-2 Cooley-Tukey, n a power of two; sign -1 forward, +1 inverse (unnormalised)
static void fft_pow2(std::vector<cd>& a, int sign)
{
	const size_t n = a.size();
	for (size_t i = 1, j = 0; i < n; ++i) {
		size_t bit = n >> 1;
		for (; j & bit; bit >>= 1) j ^= bit;
		j ^= bit;
		if (i < j) std::swap(a[i], a[j]);
	}
	for (size_t len = 2; len <= n; len <<= 1) {
		const double ang = sign * 2.0 * M_PI / (double)len;
		for (size_t i = 0; i < n; i += len)
			for (size_t k = 0; k < len / 2; ++k) {
				cd w(std::cos(ang * k), std::sin(ang * k));
				cd u = a[i + k], v = a[i + k + len / 2] * w;
				a[i + k] = u + v;
				a[i + k + len / 2] = u - v;
			}
	}
}

// exact-length DFT X_k = sum_j x_j exp(-2 pi i j k / n) for any n (Bluestein's chirp-z)
static std::vector<cd> dft(const std::vector<cd>& x)
{
	const size_t n = x.size();
	if (n == 0) return {};
	size_t m = 1;
	while (m < 2 * n - 1) m <<= 1;
	std::vector<cd> w(n), a(m, 0.0), b(m, 0.0);
	for (size_t k = 0; k < n; ++k) {
		// angle pi k^2 / n reduced modulo 2n to keep it small
		unsigned long long kk = (unsigned long long)k * k % (2ull * n);
		double ang = M_PI * (double)kk / (double)n;
		w[k] = cd(std::cos(ang), -std::sin(ang));
	}
	for (size_t k = 0; k < n; ++k) a[k] = x[k] * w[k];
	b[0] = std::conj(w[0]);
	for (size_t k = 1; k < n; ++k) b[k] = b[m - k] = std::conj(w[k]);
	fft_pow2(a, -1);
	fft_pow2(b, -1);
	for (size_t k = 0; k < m; ++k) a[k] *= b[k];
	fft_pow2(a, +1);
	std::vector<cd> X(n);
	for (size_t k = 0; k < n; ++k) X[k] = w[k] * a[k] / (double)m;
	return X;
}

} // namespace qpc

using namespace qpc;

extern "C" {

// Harmonic spectrum of one wavefunction, analysis/plot_hhs.m restated:
// d(t_i) = -z(t_i) (electron charge -1), window = sin^2(pi (t-tmin)/(tmax-tmin)) on
// (tmin, tmax), D(w_k) = DFT(d window)_k dt / (2 pi), w_k = k 2pi/(dt n), k < ceil(n/2);
// S(w) = 4 pi^2 w^2 |D|^2 / c^2 (dipole_type 1, dipole moment) or w^-2 (type 2,
// dipole acceleration), c = 137.036.  t_i = t0 + i dt.  Writes n_half = ceil(n/2)
// values to omega and spectrum.
int qpc_hhg_spectrum(const double* z, int64_t n, double t0, double dt, double tmin, double tmax, int32_t dipole_type,
	double* omega, double* spectrum)
{
	if (!z || !omega || !spectrum || n < 1 || !(dt > 0) || !(tmax > tmin) || (dipole_type != 1 && dipole_type != 2)) {
		set_error("qpc_hhg_spectrum: bad arguments");
		return QPC_ERR_ARGS;
	}
	std::vector<cd> x(n);
	for (int64_t i = 0; i < n; ++i) {
		double t = t0 + dt * (double)i;
		double win = (t > tmin && t < tmax) ? std::pow(std::sin(M_PI * (t - tmin) / (tmax - tmin)), 2) : 0.0;
		x[i] = cd(-z[i] * win, 0.0);
	}
	std::vector<cd> X = dft(x);
	const int64_t nh = (n + 1) / 2;
	const double dw = 2.0 * M_PI / (dt * (double)n), c = 137.036;
	for (int64_t k = 0; k < nh; ++k) {
		double w = dw * (double)k;
		double a = std::norm(X[k] * (dt / (2.0 * M_PI)));
		omega[k] = w;
		spectrum[k] = (dipole_type == 1 ? 4.0 * M_PI * M_PI * w * w : (w > 0 ? 4.0 * M_PI * M_PI / (w * w) : 0.0)) / (c * c) * a;
	}
	return QPC_OK;
}

// Photoelectron energy spectrum and ionization yield from projections onto the
// field-free eigenstates (eigenstate_sph::projection, population_1e.hpp:29-55):
// pes[b] = sum of |proj|^2 over states with energy in [emin + b de, emin + (b+1) de),
// de = (emax - emin)/nbins, divided by de; *bound = sum of |proj|^2 over states with
// energy < thres; *yield = 1 - *bound (ionization_sph::measure_ioyd,
// ionization_1e.hpp:15-51).  proj complex (re, im) with energy[i] its state's energy.
int qpc_pes_bin(const double* proj, const double* energy, int64_t n, double emin, double emax, int32_t nbins, double thres,
	double* pes, double* bound, double* yield)
{
	if ((n > 0 && (!proj || !energy)) || nbins < 0 || (nbins > 0 && (!pes || !(emax > emin)))) {
		set_error("qpc_pes_bin: bad arguments");
		return QPC_ERR_ARGS;
	}
	for (int b = 0; b < nbins; ++b) pes[b] = 0.0;
	const double de = nbins > 0 ? (emax - emin) / nbins : 1.0;
	double sb = 0.0;
	for (int64_t i = 0; i < n; ++i) {
		double w = proj[2 * i] * proj[2 * i] + proj[2 * i + 1] * proj[2 * i + 1];
		if (energy[i] < thres) sb += w;
		if (nbins > 0 && energy[i] >= emin && energy[i] < emax) {
			int b = (int)((energy[i] - emin) / de);
			if (b >= nbins) b = nbins - 1;
			pes[b] += w / de;
		}
	}
	if (bound) *bound = sb;
	if (yield) *yield = 1.0 - sb;
	return QPC_OK;
}

} // extern "C"
