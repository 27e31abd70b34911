// CPU oracle for the QPC-TDSE Arnoldi (Lanczos) propagator in the length gauge.
//
// TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg load this library, as the checker.  The GPU
// product never links it.
//
// It restates, in plain C++, propagator_arnoldi::propagate1 driven by
// propagator_hc_lgwz (spherical/propagator/la_1e.hpp), one step w -> exp(-i dt
// S^-1 H) w in a Krylov space of at most kmax vectors:
//   * construct_sub (la_1e.hpp:132-151): u0 = w / |w|_S, b[0] = |w|_S.
//   * multiply (la_1e.hpp:420-434): v = H_l u (symb_mul_vecd, utilities/
//     blas2.hpp:452-508) + ez y10(m,l-1) R u_{l-1} + ez y10(m,l) R u_{l+1}.
//   * orthogonalize_ip (la_1e.hpp:195-240): x_i = <u_i|v> for i < k, v = S^-1 v,
//     v -= x_i u_i (always for i = k-1, otherwise only if |x_i|^2 > 4e-27),
//     nu = <v|S|v>; nu < 1e-13 stops the expansion (b[k] = 0), else
//     v *= 1/sqrt(nu), b[k] = sqrt(nu); a[k-1] = Re x_{k-1}.
//     S^-1 is the banded Cholesky S = L L^T (LAPACK dpbtrf 'L', algorithm/
//     ed.h:182-193) followed by ltrb_inv_vecd / utrb_inv_vecd (blas2.hpp:
//     421-433, 1006-1040), applied per (m,l) channel as operator_sc::inverse_sub
//     (operators/1e.hpp:1247-1251) intends.  The shipped operator_sc::inverse_all
//     (operators/1e.hpp:1253-1260) offsets channel i by i*n_dims while stepping i
//     by n_dims, i.e. it solves blocks n_dims^2 apart; the oracle applies the
//     per-channel solve that the loop is written to perform.
//   * propagate_sub (la_1e.hpp:153-174): eigen-decomposition of the m x m
//     symmetric tridiagonal (a, b[1..m-1]) (LAPACK dstev), w_i = z_i[0]
//     exp(-i dt e_i), x_j = b[0] sum_i w_i z_i[j].  The tridiagonal eigen-solver
//     here is the implicit QL iteration with Wilkinson shifts (Bowdler, Martin,
//     Reinsch and Wilkinson, "The QR and QL algorithms for symmetric matrices",
//     Numer. Math. 11 (1968) 293-306); the step result does not depend on the
//     sign or order of the eigenvectors.
//   * eliminate_sub (la_1e.hpp:176-193): w = sum_{i<m} x_i u_i.
//   * criterion (la_1e.hpp:296-310): |x_{m-1}|^2 (0 for m = 1) > emax -> 0,
//     > emin -> 1, else 2.
// Compiled with -ffp-contract=off.
//
// Layout: state [inst][m][l][r] complex128; symmetric bands in upper-row form
// band[r*(p+1)+k] = A(r, r+k); the Cholesky factor in the same form holds
// L(r+k, r).
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <omp.h>

namespace {

using cd = std::complex<double>;

// y (=,+=) alpha * A x for symmetric band A (symb_mul_vecd, blas2.hpp:452-533)
void sbmv(int n, int p, const double* A, const cd* x, cd* y, double alpha, bool accumulate)
{
	const int m = p + 1;
	for (int i = 0; i < n; ++i) {
		int jmax = std::min(i + 1, m), kmax = std::min(m, n - i);
		const double* a = A + (long)i * m;
		cd t = 0.0;
		for (int j = 1; j < jmax; ++j) t += x[i - j] * a[-(long)j * p];
		for (int k = 0; k < kmax; ++k) t += x[i + k] * a[k];
		if (accumulate) y[i] += t * alpha;
		else y[i] = t;
	}
}

// x^H A x for symmetric band A (real part of symb_prj_vecd)
double snorm_channel(int n, int p, const double* A, const cd* x)
{
	const int m = p + 1;
	double s = 0.0;
	for (int i = 0; i < n; ++i) {
		int jmax = std::min(i + 1, m), kmax = std::min(m, n - i);
		const double* a = A + (long)i * m;
		cd t = 0.0;
		for (int j = 1; j < jmax; ++j) t += x[i - j] * a[-(long)j * p];
		for (int k = 0; k < kmax; ++k) t += x[i + k] * a[k];
		s += x[i].real() * t.real() + x[i].imag() * t.imag();
	}
	return s;
}

// u = (L L^T)^-1 u with L(r+k, r) = chol[r*(p+1)+k] (ltrb_inv_vecd then utrb_inv_vecd)
void chol_solve(int n, int p, const double* L, cd* u)
{
	const int m = p + 1;
	for (int i = 0; i < n; ++i) {
		int jmax = std::min(i + 1, m);
		cd x = u[i];
		for (int j = 1; j < jmax; ++j) x -= u[i - j] * L[(long)(i - j) * m + j];
		u[i] = x / L[(long)i * m];
	}
	for (int i = 0; i < n; ++i) {
		int s = n - 1 - i, kmax = std::min(i + 1, m);
		cd x = u[s];
		for (int k = 1; k < kmax; ++k) x -= u[s + k] * L[(long)s * m + k];
		u[s] = x / L[(long)s * m];
	}
}

// eigenvalues d[0..n) and eigenvectors (column i of z, z[j*n+i] = component j) of the
// symmetric tridiagonal with diagonal d and off-diagonal e[1..n) (e[0] unused);
// implicit QL with Wilkinson shifts.  Returns 0, or 1 if an eigenvalue failed to
// converge in 60 iterations.
int tridiag_ql(int n, double* d, double* e, double* z)
{
	for (int i = 0; i < n * n; ++i) z[i] = 0.0;
	for (int i = 0; i < n; ++i) z[i * n + i] = 1.0;
	for (int i = 1; i < n; ++i) e[i - 1] = e[i];
	if (n > 0) e[n - 1] = 0.0;
	for (int l = 0; l < n; ++l) {
		int iter = 0, mm;
		do {
			for (mm = l; mm < n - 1; ++mm) {
				double dd = std::fabs(d[mm]) + std::fabs(d[mm + 1]);
				if (std::fabs(e[mm]) <= 1e-300 || std::fabs(e[mm]) + dd == dd) break;
			}
			if (mm != l) {
				if (iter++ == 60) return 1;
				double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
				double r = std::hypot(g, 1.0);
				g = d[mm] - d[l] + e[l] / (g + (g >= 0 ? r : -r));
				double s = 1.0, c = 1.0, pp = 0.0;
				int i;
				for (i = mm - 1; i >= l; --i) {
					double f = s * e[i], b = c * e[i];
					r = std::hypot(f, g);
					e[i + 1] = r;
					if (r == 0.0) {
						d[i + 1] -= pp;
						e[mm] = 0.0;
						break;
					}
					s = f / r;
					c = g / r;
					g = d[i + 1] - pp;
					r = (d[i] - g) * s + 2.0 * c * b;
					pp = s * r;
					d[i + 1] = g + pp;
					g = c * r - b;
					for (int k = 0; k < n; ++k) {
						f = z[k * n + i + 1];
						z[k * n + i + 1] = s * z[k * n + i] + c * f;
						z[k * n + i] = c * z[k * n + i] - s * f;
					}
				}
				if (r == 0.0 && i >= l) continue;
				d[l] -= pp;
				e[l] = g;
				e[mm] = 0.0;
			}
		} while (mm != l);
	}
	return 0;
}

} // namespace

extern "C" {

struct oracle_arnoldi {
	int32_t n_r, p, n_l, n_m, m0, n_inst;
	int32_t kmax, h_per_inst;
	double dt, emin, emax;
	const double* S;    // [n_r][p+1]
	const double* chol; // [n_r][p+1], L(r+k, r)
	const double* R;    // [n_r][p+1]
	const double* H;    // [h_per_inst ? n_inst : 1][lmax+1][n_r][p+1], lmax = max|m| + n_l - 1
	const double* y10;  // [n_m][n_l], y10(m, l) couples l and l+1
};

// Banded Cholesky S = L L^T (the factor LAPACK dpbtrf 'L' returns, algorithm/ed.h:182-193),
// right-looking.  S and L in upper-row form; returns the first non-positive pivot + 1, or 0.
int oracle_chol_band(int n, int p, const double* S, double* L)
{
	const int m = p + 1;
	std::memcpy(L, S, sizeof(double) * (size_t)n * m);
	for (int j = 0; j < n; ++j) {
		double d = L[(long)j * m];
		if (!(d > 0.0)) return j + 1;
		d = std::sqrt(d);
		L[(long)j * m] = d;
		int kmax = std::min(p, n - 1 - j);
		for (int k = 1; k <= kmax; ++k) L[(long)j * m + k] /= d;
		for (int k = 1; k <= kmax; ++k) {
			double lk = L[(long)j * m + k];
			for (int q = k; q <= kmax; ++q) L[(long)(j + k) * m + (q - k)] -= lk * L[(long)j * m + q];
		}
	}
	// rows past the end of the band are zero-padded (ed.h:186-191)
	for (int j = std::max(0, n - p); j < n; ++j)
		for (int k = n - j; k <= p; ++k) L[(long)j * m + k] = 0.0;
	return 0;
}

// One Arnoldi step of every instance with ez[inst]; crit[inst] receives the criterion
// code and msub[inst] (if non-null) the Krylov dimension used.
static int arnoldi_one(const oracle_arnoldi* g, int inst, cd* w, double ez, std::vector<cd>& U, int* msub_out)
{
	const int N = g->n_r, L = g->n_l, M = g->n_m, p = g->p, K = g->kmax;
	const long nch = (long)M * L, n = nch * N, nb = (long)N * (p + 1);
	const int mmax = std::max(std::abs(g->m0), std::abs(g->m0 + M - 1));
	const double* H = g->H + (g->h_per_inst ? (long)inst * (mmax + L) * nb : 0);
	std::vector<double> a(K + 2, 0.0), b(K + 2, 0.0), z((size_t)K * K);
	std::vector<cd> x(K + 2);
	U.resize((size_t)(K + 2) * n);
	auto u = [&](int i) { return U.data() + (long)i * n; };
	// construct_sub
	double norm = 0.0;
	for (long c = 0; c < nch; ++c) norm += snorm_channel(N, p, g->S, w + c * N);
	norm = std::sqrt(norm);
	for (long e = 0; e < n; ++e) u(0)[e] = w[e] * (1.0 / norm);
	b[0] = norm;
	int msub = 0;
	bool go = true;
	while (go && msub < K) {
		const cd* u0 = u(msub);
		cd* v = u(msub + 1);
		// multiply
		for (int im = 0; im < M; ++im)
			for (int il = 0; il < L; ++il) {
				long sh = ((long)im * L + il) * N;
				long l = il + std::abs(im + g->m0);
				sbmv(N, p, H + l * nb, u0 + sh, v + sh, 0.0, false);
				if (il > 0) sbmv(N, p, g->R, u0 + sh - N, v + sh, ez * g->y10[im * L + il - 1], true);
				if (il < L - 1) sbmv(N, p, g->R, u0 + sh + N, v + sh, ez * g->y10[im * L + il], true);
			}
		const int k = ++msub;
		// orthogonalize_ip
		for (int i = 0; i < k; ++i) {
			cd s = 0.0;
			const cd* ui = u(i);
			for (long e = 0; e < n; ++e) s += std::conj(ui[e]) * v[e];
			x[i] = s;
		}
		for (long c = 0; c < nch; ++c) chol_solve(N, p, g->chol, v + c * N);
		for (int i = 0; i < k; ++i)
			if (i == k - 1 || std::norm(x[i]) > 4e-27) {
				const cd* ui = u(i);
				for (long e = 0; e < n; ++e) v[e] -= ui[e] * x[i];
			}
		double nu = 0.0;
		for (long c = 0; c < nch; ++c) nu += snorm_channel(N, p, g->S, v + c * N);
		if (nu < 1e-13) {
			nu = 0.0;
			go = false;
		} else {
			nu = std::sqrt(nu);
			for (long e = 0; e < n; ++e) v[e] *= 1.0 / nu;
		}
		a[k - 1] = x[k - 1].real();
		b[k] = nu;
	}
	// propagate_sub
	const int m = msub;
	std::vector<double> d(a.begin(), a.begin() + m), e(m + 1, 0.0), zz((size_t)m * m);
	for (int i = 1; i < m; ++i) e[i] = b[i];
	if (tridiag_ql(m, d.data(), e.data(), zz.data())) return -1;
	std::vector<cd> wv(m), xv(m, 0.0);
	for (int i = 0; i < m; ++i) wv[i] = zz[i] * std::exp(cd(0.0, -g->dt * d[i]));
	for (int j = 0; j < m; ++j) {
		cd s = 0.0;
		for (int i = 0; i < m; ++i) s += wv[i] * zz[(long)j * m + i];
		xv[j] = s * b[0];
	}
	// eliminate_sub
	for (long q = 0; q < n; ++q) {
		cd s = u(0)[q] * xv[0];
		for (int i = 1; i < m; ++i) s += u(i)[q] * xv[i];
		w[q] = s;
	}
	if (msub_out) *msub_out = m;
	double eps = m > 1 ? std::norm(xv[m - 1]) : 0.0;
	return eps > g->emax ? 0 : eps > g->emin ? 1 : 2;
}

// nt[inst] Arnoldi steps per instance with ez = ftab[inst*ld + step]; coef [inst][m][l][r];
// crit[inst*ld + step] (if non-null) the criterion code of each step, msub likewise.
// Returns 0, or 1 if a tridiagonal eigenproblem failed to converge.
int oracle_arnoldi_run(const oracle_arnoldi* g, double* coef, const double* ftab, long ld, const int64_t* nt,
	int8_t* crit, int8_t* msub, int nthreads)
{
	const long n = (long)g->n_m * g->n_l * g->n_r;
	int err = 0;
	#pragma omp parallel num_threads(nthreads) reduction(|:err)
	{
		std::vector<cd> U;
		#pragma omp for schedule(dynamic, 1)
		for (int k = 0; k < g->n_inst; ++k) {
			cd* w = (cd*)coef + (long)k * n;
			for (long s = 0; s < nt[k]; ++s) {
				int ms = 0;
				int c = arnoldi_one(g, k, w, ftab[(long)k * ld + s], U, &ms);
				if (c < 0) { err |= 1; break; }
				if (crit) crit[(long)k * ld + s] = (int8_t)c;
				if (msub) msub[(long)k * ld + s] = (int8_t)ms;
			}
		}
	}
	return err;
}

// absorber_mask::operator() (absorber.hpp:51-63): per channel w = S^-1 (M w), the band
// product by symb_mul_vecd and the Cholesky solves by ltrb_inv_vecd / utrb_inv_vecd.
void oracle_mask(int n_r, int p, long n_ch, const double* M, const double* chol, double* coef)
{
	std::vector<cd> t(n_r);
	for (long c = 0; c < n_ch; ++c) {
		cd* w = (cd*)coef + c * n_r;
		sbmv(n_r, p, M, w, t.data(), 0.0, false);
		chol_solve(n_r, p, chol, t.data());
		for (int r = 0; r < n_r; ++r) w[r] = t[r];
	}
}

} // extern "C"

