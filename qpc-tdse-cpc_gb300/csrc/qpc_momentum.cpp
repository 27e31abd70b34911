// Host tables of the photoelectron momentum spectra: the projection onto Coulomb
// (or plane) partial waves of spectrum_c_pcs and the surface quantities of the
// t-SURFF flux integral of spectrum_c_tsf (spherical/spectrum/momentum_1e.hpp:1-228,
// 443-514, 778-866).  The GPU applies them (qpc_momentum.cu).
//
// Special functions, each from a published method:
//   * Coulomb wave functions F_l(eta, rho), F'_l (Abramowitz & Stegun ch. 14
//     normalisation, Wronskian F'G - FG' = 1) by Steed's method (A. R. Barnett,
//     Comput. Phys. Commun. 27 (1982) 147): CF1 for F'/F at l_max, downward
//     recurrence, and the absolute value at l = 0 from CF2 for H+'/H+ with the
//     Wronskian, or from the power series A&S 14.1.3-14.1.8 near the origin;
//   * Coulomb phase sigma_l = arg Gamma(l + 1 + i eta): Stirling's series for
//     ln Gamma (A&S 6.1.41) after shifting the argument, then A&S 14.5.6;
//   * normalised associated Legendre functions with the Condon-Shortley phase
//     (Y_lm(theta, 0)) by the standard three-term recurrence in l;
//   * partial waves of screened potentials: the radial equation integrated by the
//     Dormand-Prince 5(4) pair and matched to F_l, G_l at the asymptotic radius.
#include "qpc_internal.h"
#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <thread>
#include <vector>

namespace qpc {
namespace {

const double PI = 3.14159265358979323846;

// arg Gamma(1 + i eta): ln Gamma(z) = ln Gamma(z + N) - sum_{j<N} ln(z + j) with Stirling's
// series for ln Gamma(z + N), |z + N| >= 17, carried in long double.
long double coulomb_sigma0(double eta)
{
	typedef std::complex<long double> cl;
	const int N = 16;
	long double im = 0;
	for (int j = 0; j < N; ++j) im -= std::atan2((long double)eta, 1.0L + j);
	cl w(1.0L + N, (long double)eta);
	static const long double B2k[] = {1.0L / 6, -1.0L / 30, 1.0L / 42, -1.0L / 30, 5.0L / 66, -691.0L / 2730, 7.0L / 6, -3617.0L / 510};
	cl lg = (w - 0.5L) * std::log(w) - w;
	cl wp = w, w2 = w * w;
	for (int k = 1; k <= 8; ++k) {
		lg += B2k[k - 1] / ((long double)(2 * k) * (2 * k - 1) * wp);
		wp *= w2;
	}
	return im + lg.imag();
}

// F_0(eta, rho), F_0' by the power series F_0 = C_0 sum_{k>=1} A_k rho^k, A_1 = 1, A_2 = eta,
// k (k-1) A_k = 2 eta A_{k-1} - A_{k-2}, C_0^2 = 2 pi eta / (exp(2 pi eta) - 1).
void coulomb_series0(double eta, double rho, double& f, double& fp)
{
	long double c0 = eta == 0.0 ? 1.0L : std::sqrt(2.0L * PI * eta / std::expm1(2.0L * PI * eta));
	long double a2 = 1.0L, a1 = (long double)eta;	// A_{k-2}, A_{k-1} for k = 3
	long double rk = (long double)rho * rho;	// rho^(k-1) for k = 3
	long double s = rho + (long double)eta * rho * rho, sp = 1.0L + 2.0L * eta * rho;
	bool small_prev = false;	// A_k can vanish for every other k (eta = 0): stop after two small terms in a row
	for (int k = 3; k < 20000; ++k) {
		long double ak = (2.0L * eta * a1 - a2) / ((long double)k * (k - 1));
		long double t = ak * rk * rho, tp = k * ak * rk;
		s += t; sp += tp;
		a2 = a1; a1 = ak; rk *= rho;
		const bool small = std::fabs(t) <= 1e-21L * std::fabs(s) && std::fabs(tp) <= 1e-21L * std::fabs(sp);
		if (k > 8 && small && small_prev) break;
		small_prev = small;
	}
	f = (double)(c0 * s);
	fp = (double)(c0 * sp);
}

// p + i q = H+'/H+ at l = 0 (Steed's CF2): i (1 - eta/rho) + (i/rho) K with
// K = a_1/(b_1 + a_2/(b_2 + ...)), a_n = (n + i eta)(n - 1 + i eta), b_n = 2 (rho - eta + i n),
// by the modified Lentz method.  Returns the iterations used, or -1 without convergence.
int coulomb_cf2(double eta, double rho, double& p, double& q)
{
	typedef std::complex<double> cd;
	const double tiny = 1e-300;
	cd f(tiny, 0.0), C = f, D(0.0, 0.0);
	const int maxit = 200000;
	int n = 1;
	for (; n <= maxit; ++n) {
		cd a = cd(n, eta) * cd(n - 1, eta), b(2.0 * (rho - eta), 2.0 * n);
		D = b + a * D;
		if (D == cd(0.0, 0.0)) D = tiny;
		C = b + a / C;
		if (C == cd(0.0, 0.0)) C = tiny;
		D = 1.0 / D;
		cd del = C * D;
		f *= del;
		if (std::abs(del - 1.0) < 1e-16) break;
	}
	if (n > maxit) return -1;
	cd pq = cd(0.0, 1.0 - eta / rho) + cd(0.0, 1.0 / rho) * f;
	p = pq.real(); q = pq.imag();
	return n;
}

}  // namespace

// F[l] = F_l(eta, rho), Fp[l] = dF_l/drho for l = 0..lmax, rho > 0.  Returns 0, or a positive
// count of continued fractions that did not converge.
int coulomb_f(double eta, double rho, int lmax, double* F, double* Fp)
{
	int bad = 0;
	const int L = lmax;
	// CF1 at l = L: F'_L/F_L = S_{L+1} - R_{L+1}^2/(T_{L+1} - R_{L+2}^2/(T_{L+2} - ...)),
	// S_l = l/rho + eta/l, R_l^2 = 1 + eta^2/l^2, T_l = S_l + S_{l+1}.  The product of the signs of the
	// Lentz denominators is the sign of F_L.
	const double tiny = 1e-300;
	double f = (L + 1) / rho + eta / (L + 1);
	if (f == 0.0) f = tiny;
	double C = f, D = 0.0;
	int sgn = 1;
	const long maxit = 20000 + 4 * (long)rho;
	long j = 1;
	for (; j <= maxit; ++j) {
		const double l = L + j;
		const double a = -(1.0 + eta * eta / (l * l)), b = (2 * l + 1) * (1.0 / rho + eta / (l * (l + 1)));
		D = b + a * D;
		if (D == 0.0) D = tiny;
		C = b + a / C;
		if (C == 0.0) C = tiny;
		D = 1.0 / D;
		const double del = C * D;
		f *= del;
		if (D < 0) sgn = -sgn;
		if (std::fabs(del - 1.0) < 1e-16) break;
	}
	if (j > maxit) ++bad;
	// downward recurrence, rescaled so that nothing overflows on the way to l = 0
	F[L] = sgn;
	Fp[L] = f * sgn;
	for (int l = L; l >= 1; --l) {
		const double S = l / rho + eta / l, R = std::sqrt(1.0 + (eta / l) * (eta / l));
		F[l - 1] = (S * F[l] + Fp[l]) / R;
		Fp[l - 1] = S * F[l - 1] - R * F[l];
		if (std::fabs(F[l - 1]) > 1e250 || std::fabs(Fp[l - 1]) > 1e250)
			for (int k = l - 1; k <= L; ++k) { F[k] *= 1e-250; Fp[k] *= 1e-250; }
	}
	// absolute value at l = 0
	double scale;
	// the series near the origin, and for a repulsive field (eta > 0) inside the l = 0 turning
	// point 2 eta, where its terms share one sign and CF2 loses accuracy
	if ((rho < 1.0 && rho * std::fabs(eta) < 2.0) || (eta > 0.0 && rho < 1.8 * eta)) {
		double f0, f0p;
		coulomb_series0(eta, rho, f0, f0p);
		scale = std::fabs(F[0]) > std::fabs(Fp[0]) ? f0 / F[0] : f0p / Fp[0];
	} else {
		double p, q;
		if (coulomb_cf2(eta, rho, p, q) < 0) ++bad;
		const double g = Fp[0] / F[0];
		const double amp = std::sqrt(q / ((g - p) * (g - p) + q * q));
		scale = amp / std::fabs(F[0]);
	}
	for (int l = 0; l <= L; ++l) { F[l] *= scale; Fp[l] *= scale; }
	return bad;
}

// sigma[l] = arg Gamma(l + 1 + i eta), l = 0..lmax (A&S 14.5.6: sigma_l = sigma_{l-1} + atan(eta/l))
void coulomb_sigma(double eta, int lmax, double* sigma)
{
	long double s = coulomb_sigma0(eta);
	sigma[0] = (double)s;
	for (int l = 1; l <= lmax; ++l) {
		s += std::atan((long double)eta / l);
		sigma[l] = (double)s;
	}
}

// Y_lm(theta, 0) for 0 <= m <= l <= lmax at x = cos(theta), out[l*(l+1)/2 + m]: the spherical-harmonic
// normalisation sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!) P_l^m(x) with the Condon-Shortley phase (-1)^m.
void sph_legendre(int lmax, double x, double* out)
{
	const double s = std::sqrt(std::max(0.0, (1.0 - x) * (1.0 + x)));
	double pmm = std::sqrt(1.0 / (4.0 * PI));	// Y_00
	for (int m = 0; m <= lmax; ++m) {
		if (m > 0) pmm *= -s * std::sqrt((2.0 * m + 1.0) / (2.0 * m));
		out[m * (m + 1) / 2 + m] = pmm;
		if (m == lmax) break;
		double p1 = x * std::sqrt(2.0 * m + 3.0) * pmm;	// Y_{m+1, m}
		out[(m + 1) * (m + 2) / 2 + m] = p1;
		double p0 = pmm;
		for (int l = m + 2; l <= lmax; ++l) {
			const double a = std::sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
			const double b = std::sqrt(((double)(l - 1) * (l - 1) - (double)m * m) / (4.0 * (l - 1) * (l - 1) - 1.0));
			const double p2 = a * (x * p1 - b * p0);
			out[l * (l + 1) / 2 + m] = p2;
			p0 = p1; p1 = p2;
		}
	}
}

// F, F', G, G' for l = 0..lmax at rho where Steed's CF2 applies (rho >= 1, outside a repulsive
// turning point): F as coulomb_f, G_0 = (F_0' - p F_0)/q, G_0' = p G_0 - q F_0 from p + iq = H+'/H+,
// then G upward (A&S 14.2.1-2), the stable direction for the irregular solution.
int coulomb_fg(double eta, double rho, int lmax, double* F, double* Fp, double* G, double* Gp)
{
	if (!(rho >= 1.0) || (eta > 0.0 && rho < 1.8 * eta)) return 1;
	int bad = coulomb_f(eta, rho, lmax, F, Fp);
	double p, q;
	if (coulomb_cf2(eta, rho, p, q) < 0) ++bad;
	G[0] = (Fp[0] - p * F[0]) / q;
	Gp[0] = p * G[0] - q * F[0];
	for (int l = 0; l < lmax; ++l) {
		const double L = l + 1, S = L / rho + eta / L, R = std::sqrt(1.0 + (eta / L) * (eta / L));
		G[l + 1] = (S * G[l] - Gp[l]) / R;
		Gp[l + 1] = R * G[l] - S * G[l + 1];
	}
	return bad;
}

namespace {

// u'' = -(1 - 2 e0/x - l(l+1)/x^2 - 2 e1 e^{d1 x}/x) u in x = k r for V = -(Z + a e^{-s r})/r and mass m:
// e0 = -m Z/k, e1 = -m a/k, d1 = -s/k (the scaled radial equation of equation_hydrogenic_yukawa,
// spherical/spectrum/equation.hpp:66-123).
struct radial_ode {
	double e0, e1, d1, ll;
	void operator()(double x, const double* y, double* dy) const
	{
		const double g = 1.0 - 2.0 * e0 / x - ll / (x * x) - (e1 != 0.0 ? 2.0 * e1 * std::exp(d1 * x) / x : 0.0);
		dy[0] = y[1];
		dy[1] = -g * y[0];
	}
};

// Dormand-Prince 5(4) (J. R. Dormand, P. J. Prince, J. Comput. Appl. Math. 6 (1980) 19) from x0 to x1 with
// step control on the relative error max|err| / (rtol max|y|); h carries the step size between calls.
// Returns 0, or 1 if the step count ran out.
int dopri(const radial_ode& f, double* y, double x0, double x1, double& h, double rtol)
{
	static const double c2 = 1.0 / 5, c3 = 3.0 / 10, c4 = 4.0 / 5, c5 = 8.0 / 9;
	static const double a21 = 1.0 / 5, a31 = 3.0 / 40, a32 = 9.0 / 40, a41 = 44.0 / 45, a42 = -56.0 / 15, a43 = 32.0 / 9;
	static const double a51 = 19372.0 / 6561, a52 = -25360.0 / 2187, a53 = 64448.0 / 6561, a54 = -212.0 / 729;
	static const double a61 = 9017.0 / 3168, a62 = -355.0 / 33, a63 = 46732.0 / 5247, a64 = 49.0 / 176, a65 = -5103.0 / 18656;
	static const double b1 = 35.0 / 384, b3 = 500.0 / 1113, b4 = 125.0 / 192, b5 = -2187.0 / 6784, b6 = 11.0 / 84;
	static const double e1 = 71.0 / 57600, e3 = -71.0 / 16695, e4 = 71.0 / 1920, e5 = -17253.0 / 339200, e6 = 22.0 / 525, e7 = -1.0 / 40;
	double x = x0;
	if (x1 <= x0) return 0;
	if (!(h > 0.0)) h = std::min(x1 - x0, 1e-3 * std::max(1.0, x0));
	double k1[2], k2[2], k3[2], k4[2], k5[2], k6[2], k7[2], t[2], yn[2];
	f(x, y, k1);
	for (long it = 0; it < 10000000; ++it) {
		if (x >= x1) return 0;
		const bool last = x + h >= x1;
		const double hh = last ? x1 - x : h;
		for (int i = 0; i < 2; ++i) t[i] = y[i] + hh * a21 * k1[i];
		f(x + c2 * hh, t, k2);
		for (int i = 0; i < 2; ++i) t[i] = y[i] + hh * (a31 * k1[i] + a32 * k2[i]);
		f(x + c3 * hh, t, k3);
		for (int i = 0; i < 2; ++i) t[i] = y[i] + hh * (a41 * k1[i] + a42 * k2[i] + a43 * k3[i]);
		f(x + c4 * hh, t, k4);
		for (int i = 0; i < 2; ++i) t[i] = y[i] + hh * (a51 * k1[i] + a52 * k2[i] + a53 * k3[i] + a54 * k4[i]);
		f(x + c5 * hh, t, k5);
		for (int i = 0; i < 2; ++i) t[i] = y[i] + hh * (a61 * k1[i] + a62 * k2[i] + a63 * k3[i] + a64 * k4[i] + a65 * k5[i]);
		f(x + hh, t, k6);
		for (int i = 0; i < 2; ++i) yn[i] = y[i] + hh * (b1 * k1[i] + b3 * k3[i] + b4 * k4[i] + b5 * k5[i] + b6 * k6[i]);
		f(x + hh, yn, k7);
		double err = 0.0;
		const double sc = rtol * std::max(std::max(std::fabs(y[0]), std::fabs(y[1])), std::max(std::fabs(yn[0]), std::fabs(yn[1]))) + 1e-300;
		for (int i = 0; i < 2; ++i)
			err = std::max(err, std::fabs(hh * (e1 * k1[i] + e3 * k3[i] + e4 * k4[i] + e5 * k5[i] + e6 * k6[i] + e7 * k7[i])) / sc);
		if (err <= 1.0) {
			x = last ? x1 : x + hh;
			y[0] = yn[0]; y[1] = yn[1];
			k1[0] = k7[0]; k1[1] = k7[1];
			if (!last) h = hh * std::min(5.0, 0.9 * std::pow(std::max(err, 1e-10), -0.2));
		} else {
			h = hh * std::max(0.2, 0.9 * std::pow(err, -0.2));
		}
	}
	return 1;
}

}  // namespace

// The regular partial wave of V = -(Z + a e^{-s r})/r at x_i = k r_i (ascending), normalised so that
// asymptotically u = cos(delta) F_l(eta) + sin(delta) G_l(eta), eta = -m Z/k (the solution::initialize
// of spherical/spectrum/equation.hpp:367-421): started from F_l(-m (Z + a)/k, x) near the origin,
// integrated through the points to the asymptotic radius max(eta^2 + l, 100, 32 k/s), and matched there
// to F, G.  *Delta = delta + sigma_l reduced into (-pi/2, pi/2] with the sign carried by u, as the
// reference's arctangent leaves it.  Returns 0 or a positive error count.
int coulomb_partial_wave(double Z, double a, double s, double mass, double k, int l, const double* x, int n, double* u, double* Delta)
{
	radial_ode f{-mass * Z / k, -mass * a / k, -s / k, (double)l * (l + 1)};
	const double rtol = 5e-11;
	int bad = 0;
	std::vector<double> F(l + 1), Fp(l + 1), G(l + 1), Gp(l + 1);
	double y[2];
	const double xin = l == 0 ? 1e-7 : 5e-7 * (l + 1) * l;
	double x0 = x[0] < xin ? x[0] : xin;
	if (coulomb_f(f.e0 + f.e1, x0, l, F.data(), Fp.data())) ++bad;
	y[0] = F[l]; y[1] = Fp[l];
	double h = 0.0;	// u and y share one scale, lowered together when the solution grows
	for (int i = 0; i < n; ++i) {
		if (dopri(f, y, x0, x[i], h, rtol)) ++bad;
		x0 = x[i];
		if (std::fabs(y[0]) > 1e150 || std::fabs(y[1]) > 1e150) {
			for (int j = 0; j < i; ++j) u[j] *= 1e-290;
			y[0] *= 1e-290; y[1] *= 1e-290;
		}
		u[i] = y[0];
	}
	const double large = std::max(std::max(f.e0 * f.e0 + l, 100.0), s != 0.0 ? 32.0 * k / s : 0.0);
	const double eta = s != 0.0 ? f.e0 : f.e0 + f.e1;
	if (x0 < large) {
		if (dopri(f, y, x0, large, h, rtol)) ++bad;
		x0 = large;
	}
	if (coulomb_fg(eta, x0, l, F.data(), Fp.data(), G.data(), Gp.data())) ++bad;
	// y = A (c F + s G): u F' - u' F = A s, u' G - u G' = A c  (Wronskian F'G - FG' = 1)
	const double As = y[0] * Fp[l] - y[1] * F[l], Ac = y[1] * G[l] - y[0] * Gp[l];
	const double delta = std::atan2(As, Ac);
	std::vector<double> sig(l + 1);
	coulomb_sigma(eta, l, sig.data());
	double D = delta + sig[l];
	D = std::remainder(D, PI);	// into [-pi/2, pi/2]
	if (D <= -0.5 * PI) D += PI;
	// normalisation with the reduced phase: nm y = cos(D - sigma) F + sin(D - sigma) G at x0
	const double c = std::cos(D - sig[l]), sn = std::sin(D - sig[l]);
	const double nm = std::fabs(y[0]) >= std::fabs(y[1]) ? (c * F[l] + sn * G[l]) / y[0] : (c * Fp[l] + sn * Gp[l]) / y[1];
	for (int i = 0; i < n; ++i) u[i] *= nm;
	*Delta = D;
	return bad;
}

}  // namespace qpc

using namespace qpc;

namespace {

int dims_ok(const qpc_dims* d)
{
	return d && d->n_r >= 2 * d->p + 2 && d->p >= 1 && d->p <= QPC_MAX_RANK && d->n_l >= 1 && d->n_m >= 1;
}

int lmax_of(const qpc_dims* d)
{
	const int m1 = d->m0 + d->n_m - 1;
	return std::max(std::abs(d->m0), std::abs(m1)) + d->n_l - 1;
}

// set_sequence_lin / set_sequence_sqr (spherical/spectrum/inventory.h:15-39)
void seq_lin(double* a, double x0, double x1, int n)
{
	const double dx = (x1 - x0) / (n > 1 ? n - 1 : 1);
	for (int i = 0; i < n; ++i) a[i] = i * dx + x0;
	if (n > 1) a[n - 1] = x1;
}
void seq_sqr(double* a, double x0, double x1, int n)
{
	const double dx = (x1 - x0) / (n > 1 ? n - 1 : 1);
	for (int i = 0; i < n; ++i) a[i] = std::sqrt(2.0 * (i * dx + x0));
	if (n > 1) a[n - 1] = std::sqrt(2.0 * x1);
}

int axes(const qpc_kgrid* g, double* kr, double* kt, double* kp)
{
	if (!g || g->nkr < 1 || g->nkt < 1 || g->nkp < 1 || (g->flag != 0 && g->flag != 1)) return QPC_ERR_ARGS;
	seq_lin(kp, g->kpmin, g->kpmax, g->nkp);
	seq_lin(kt, g->ktmin, g->ktmax, g->nkt);
	if (g->flag == 0) seq_lin(kr, g->krmin, g->krmax, g->nkr);
	else seq_sqr(kr, 0.5 * g->krmin * g->krmin, 0.5 * g->krmax * g->krmax, g->nkr);
	for (int i = 0; i < g->nkr; ++i) if (!(kr[i] > 0.0) || !std::isfinite(kr[i])) return QPC_ERR_ARGS;
	return QPC_OK;
}

// plm[kt][im][il] = Y_lm(kt, 0) with Y_l,-m = (-1)^m Y_lm (the legendre::get of
// functions/basis_legendre.h:55-58), exm[kp][im] = exp(i m kp) (initialize_ph / initialize_th,
// momentum_1e.hpp:11-50)
void angular(const qpc_dims* d, int nkt, const double* kt, int nkp, const double* kp, double* plm, double* exm)
{
	const int lmax = lmax_of(d);
	std::vector<double> y((size_t)(lmax + 1) * (lmax + 2) / 2);
	for (int it = 0; it < nkt; ++it) {
		sph_legendre(lmax, std::cos(kt[it]), y.data());
		for (int im = 0; im < d->n_m; ++im) {
			const int m = d->m0 + im, am = std::abs(m);
			for (int il = 0; il < d->n_l; ++il) {
				const int l = am + il;
				const double v = y[(size_t)l * (l + 1) / 2 + am];
				plm[((size_t)it * d->n_m + im) * d->n_l + il] = (m < 0 && (am & 1)) ? -v : v;
			}
		}
	}
	for (int ip = 0; ip < nkp; ++ip)
		for (int im = 0; im < d->n_m; ++im) {
			const double a = (d->m0 + im) * kp[ip];
			exm[2 * ((size_t)ip * d->n_m + im)] = std::cos(a);
			exm[2 * ((size_t)ip * d->n_m + im) + 1] = std::sin(a);
		}
}

int basis_from(const qpc_dims* d, const double* knots, radial_basis& B)
{
	B.n = d->n_r; B.p = d->p; B.nq = 2 * d->p + 2;
	B.t.assign(knots, knots + d->n_r + d->p + 3);
	for (size_t i = 1; i < B.t.size(); ++i) if (!(B.t[i] >= B.t[i - 1])) return QPC_ERR_ARGS;
	build_basis(B);
	return QPC_OK;
}

}  // namespace

extern "C" {

int qpc_coulomb_f(double eta, double rho, int32_t lmax, double* F, double* Fp)
{
	if (lmax < 0 || !(rho > 0.0) || !std::isfinite(rho) || !std::isfinite(eta) || !F || !Fp) return QPC_ERR_ARGS;
	return coulomb_f(eta, rho, lmax, F, Fp) ? QPC_ERR_NUMERIC : QPC_OK;
}

int qpc_coulomb_sigma(double eta, int32_t lmax, double* sigma)
{
	if (lmax < 0 || !std::isfinite(eta) || !sigma) return QPC_ERR_ARGS;
	coulomb_sigma(eta, lmax, sigma);
	return QPC_OK;
}

int qpc_sph_legendre(int32_t lmax, double x, double* out)
{
	if (lmax < 0 || !(x >= -1.0 && x <= 1.0) || !out) return QPC_ERR_ARGS;
	sph_legendre(lmax, x, out);
	return QPC_OK;
}

// spectrum_c_pcs::initialize with the analytic Coulomb waves (momentum_1e.hpp:453-485, initialize_kr
// 119-148): ijl[kr][l][j] = int B_j(r) F_l(-zc/k, k r) w(r) dr / k by the radial quadrature, with
// w = 1/(1 + exp(-5 (r - rb))) for rb > 0 (the plane-wave projection) and w = 1 otherwise;
// cps[kr][l] = exp(i (sigma_l - l pi/2)).
int qpc_pcs_tables(const qpc_dims* d, const double* knots, const qpc_kgrid* g, double zc, double rb, double* kr, double* kt,
	double* kp, double* ijl, double* plm, double* exm, double* cps)
{
	if (!dims_ok(d) || !knots || !kr || !kt || !kp || !ijl || !plm || !exm || !cps || !std::isfinite(zc) || !std::isfinite(rb))
		return QPC_ERR_ARGS;
	int rc = axes(g, kr, kt, kp);
	if (rc) return rc;
	radial_basis B;
	if ((rc = basis_from(d, knots, B))) return rc;
	angular(d, g->nkt, kt, g->nkp, kp, plm, exm);
	const int lmax = lmax_of(d), nl = lmax + 1, n = d->n_r, p = d->p, nq = B.nq, ni = B.nint();
	std::atomic<int> next(0), bad(0);
	auto work = [&]() {
		std::vector<double> F((size_t)nl * ni * nq, 0.0), f(nl), fp(nl), sig(nl);
		for (int ik; (ik = next.fetch_add(1)) < g->nkr;) {
			const double k = kr[ik], eta = -zc / k;
			for (int s = p; s < ni - p; ++s)
				for (int q = 0; q < nq; ++q) {
					const double x = B.xq[(size_t)s * nq + q];
					if (!(B.wq[(size_t)s * nq + q] != 0.0) || !(x > 0.0)) continue;
					if (coulomb_f(eta, k * x, lmax, f.data(), fp.data())) bad.fetch_add(1);
					const double w = rb > 0.0 ? 1.0 / (1.0 + std::exp(-5.0 * (x - rb))) : 1.0;
					for (int l = 0; l < nl; ++l) F[((size_t)l * ni + s) * nq + q] = f[l] * w;
				}
			for (int l = 0; l < nl; ++l)
				for (int j = 0; j < n; ++j) {
					// absolute spline a = j + 1 lives on intervals a .. a + p
					const int a = j + 1;
					double acc = 0.0;
					for (int s = a; s <= a + p; ++s) {
						if (s < p || s >= ni - p) continue;
						const int jj = a - (s - p);
						for (int q = 0; q < nq; ++q)
							acc += B.wq[(size_t)s * nq + q] * F[((size_t)l * ni + s) * nq + q] * B.b0[((size_t)s * (p + 1) + jj) * nq + q];
					}
					ijl[((size_t)ik * nl + l) * n + j] = acc / k;
				}
			coulomb_sigma(eta, lmax, sig.data());
			for (int l = 0; l < nl; ++l) {
				const double ph = sig[l] - l * PI / 2.0;
				cps[2 * ((size_t)ik * nl + l)] = std::cos(ph);
				cps[2 * ((size_t)ik * nl + l) + 1] = std::sin(ph);
			}
		}
	};
	unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
	nt = std::min<unsigned>(nt, (unsigned)g->nkr);
	std::vector<std::thread> th;
	for (unsigned i = 1; i < nt; ++i) th.emplace_back(work);
	work();
	for (auto& t : th) t.join();
	if (bad.load()) { set_error("Coulomb continued fraction did not converge at %d points", bad.load()); return QPC_ERR_NUMERIC; }
	return QPC_OK;
}

// spectrum_c_pcs::initialize with numerical partial waves (momentum_1e.hpp:487-512, initialize_kr 150-188,
// the "numerical PCS" the driver picks for screened potentials, binsrc/sphTDSE.cpp:313-316, 340-342):
// for V = -(zc + zs e^{-sigma r})/r and mass 1, u_l(k r) from coulomb_partial_wave on the quadrature
// points, ijl[kr][l][r] = int B_r u_l dr / k, cps[kr][l] = e^{i (Delta_l - l pi/2)}; the other tables as
// qpc_pcs_tables.
int qpc_pcs_tables_numeric(const qpc_dims* d, const double* knots, const qpc_kgrid* g, const qpc_potential* pot, double* kr,
	double* kt, double* kp, double* ijl, double* plm, double* exm, double* cps)
{
	if (!dims_ok(d) || !knots || !pot || !kr || !kt || !kp || !ijl || !plm || !exm || !cps) return QPC_ERR_ARGS;
	const double Z = pot->zc, A = pot->kind == QPC_POTENTIAL_YUKAWA ? pot->zs : 0.0, sg = pot->kind == QPC_POTENTIAL_YUKAWA ? pot->sigma : 0.0;
	if (!std::isfinite(Z) || !std::isfinite(A) || !(sg >= 0.0) || (A != 0.0 && !(sg > 0.0))) return QPC_ERR_ARGS;
	int rc = axes(g, kr, kt, kp);
	if (rc) return rc;
	radial_basis B;
	if ((rc = basis_from(d, knots, B))) return rc;
	angular(d, g->nkt, kt, g->nkp, kp, plm, exm);
	const int lmax = lmax_of(d), nl = lmax + 1, n = d->n_r, p = d->p, nq = B.nq, ni = B.nint();
	// the quadrature points with weight, ascending
	std::vector<int> pidx;
	for (int s = p; s < ni - p; ++s)
		for (int q = 0; q < nq; ++q)
			if (B.wq[(size_t)s * nq + q] != 0.0 && B.xq[(size_t)s * nq + q] > 0.0) pidx.push_back(s * nq + q);
	const int np = (int)pidx.size();
	std::atomic<int> next(0), bad(0);
	auto work = [&]() {
		std::vector<double> x(np), u(np), F((size_t)ni * nq, 0.0);
		for (int job; (job = next.fetch_add(1)) < g->nkr * nl;) {
			const int ik = job / nl, l = job % nl;
			const double k = kr[ik];
			for (int i = 0; i < np; ++i) x[i] = k * B.xq[pidx[i]];
			double D = 0.0;
			if (coulomb_partial_wave(Z, A, sg, 1.0, k, l, x.data(), np, u.data(), &D)) bad.fetch_add(1);
			for (int i = 0; i < np; ++i) F[pidx[i]] = u[i];
			for (int j = 0; j < n; ++j) {
				const int a = j + 1;
				double acc = 0.0;
				for (int s = a; s <= a + p; ++s) {
					if (s < p || s >= ni - p) continue;
					const int jj = a - (s - p);
					for (int q = 0; q < nq; ++q)
						acc += B.wq[(size_t)s * nq + q] * F[(size_t)s * nq + q] * B.b0[((size_t)s * (p + 1) + jj) * nq + q];
				}
				ijl[((size_t)ik * nl + l) * n + j] = acc / k;
			}
			const double ph = D - l * PI / 2.0;
			cps[2 * ((size_t)ik * nl + l)] = std::cos(ph);
			cps[2 * ((size_t)ik * nl + l) + 1] = std::sin(ph);
		}
	};
	unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
	std::vector<std::thread> th;
	for (unsigned i = 1; i < nt; ++i) th.emplace_back(work);
	work();
	for (auto& t : th) t.join();
	if (bad.load()) { set_error("partial-wave integration failed for %d (k, l)", bad.load()); return QPC_ERR_NUMERIC; }
	return QPC_OK;
}

// spectrum_c_tsf::initialize (momentum_1e.hpp:778-866): the splines non-zero at r0 with their values
// b0 and derivatives br (ib: active index), j0[kr][l] = F_l(-zc/k, k r0)/k and jr[kr][l] = F'_l(-zc/k, k r0),
// y0[kt][im][il] = Y_lm(kt, 0), e0[kp][im] = exp(i m kp), and the angular elements
// pmat[0] = <l m|cos|l+1 m>, pmat[1] = <l m|sin e^-i phi|l+1 m+1>, pmat[2] = <l m|sin e^-i phi|l-1 m+1>
// per (im, il) (integrate_cos, integrate_sinexp1/2, spherical/utilities/basisfunc.hpp:222-259).
int qpc_tsurff_tables(const qpc_dims* d, const double* knots, const qpc_kgrid* g, double r0, double zc, double* kr, double* kt,
	double* kp, int32_t* nb, int32_t* ib, double* b0, double* br, double* j0, double* jr, double* y0, double* e0, double* pmat)
{
	if (!dims_ok(d) || !knots || !kr || !kt || !kp || !nb || !ib || !b0 || !br || !j0 || !jr || !y0 || !e0 || !pmat || !std::isfinite(zc))
		return QPC_ERR_ARGS;
	int rc = axes(g, kr, kt, kp);
	if (rc) return rc;
	const int n = d->n_r, p = d->p, lmax = lmax_of(d), nl = lmax + 1;
	std::vector<double> t(knots, knots + n + p + 3);
	for (size_t i = 1; i < t.size(); ++i) if (!(t[i] >= t[i - 1])) return QPC_ERR_ARGS;
	if (!(r0 > t.front() && r0 < t.back())) return QPC_ERR_ARGS;
	// interval [t_s, t_s+1) holding r0
	int s = p;
	for (int i = p; i < (int)t.size() - 1; ++i) if (t[i] <= r0 && r0 < t[i + 1]) { s = i; break; }
	std::vector<double> v0(p + 1), v1(p + 1);
	bspline_eval(t, s, p, r0, v0.data(), v1.data());
	int cnt = 0;
	for (int jj = 0; jj <= p; ++jj) {
		const int a = s - p + jj, i = a - 1;	// absolute spline a, active index a - 1
		if (i < 0 || i >= n || !(v0[jj] > 0.0)) continue;
		ib[cnt] = i; b0[cnt] = v0[jj]; br[cnt] = v1[jj]; ++cnt;
	}
	*nb = cnt;
	std::vector<double> f(nl), fp(nl);
	for (int ik = 0; ik < g->nkr; ++ik) {
		const double k = kr[ik];
		if (coulomb_f(-zc / k, k * r0, lmax, f.data(), fp.data())) { set_error("Coulomb continued fraction did not converge"); return QPC_ERR_NUMERIC; }
		for (int l = 0; l < nl; ++l) { j0[(size_t)ik * nl + l] = f[l] / k; jr[(size_t)ik * nl + l] = fp[l]; }
	}
	angular(d, g->nkt, kt, g->nkp, kp, y0, e0);
	const size_t nch = (size_t)d->n_m * d->n_l;
	for (int im = 0; im < d->n_m; ++im)
		for (int il = 0; il < d->n_l; ++il) {
			const long m = d->m0 + im, l = std::labs(m) + il;
			const size_t c = (size_t)im * d->n_l + il;
			pmat[c] = std::sqrt(double((l + 1) * (l + 1) - m * m) / double((2 * l + 1) * (2 * l + 3)));
			pmat[nch + c] = -std::sqrt(double((l + m + 2) * (l + m + 1)) / double((2 * l + 1) * (2 * l + 3)));
			pmat[2 * nch + c] = +std::sqrt(double((l - m) * (l - m - 1)) / double((2 * l + 1) * (2 * l - 1)));
		}
	return QPC_OK;
}

}  // extern "C"
