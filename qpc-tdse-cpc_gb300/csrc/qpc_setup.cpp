// Host-side setup for the GB300 propagation engine: radial B-spline matrices,
// the angular coupling eigensystem, Crank-Nicolson band factorisation, field-free
// eigenstates and laser-field tables.  This is the one-time work the reference
// does on the CPU before its step loop (binsrc/sphTDSE.cpp:742-776); the time
// stepping itself runs on the GPU (qpc_engine.cu).
//
// Band storage follows the reference: a symmetric banded matrix with half
// bandwidth p is kept as band[r*(p+1)+k] = A(r, r+k) for k = 0..p
// (spherical/operators/1e.hpp:20).  Entries with r+k >= n are stored as 0.
#include "qpc_internal.h"
#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>

namespace qpc {

// ------------------------------------------------------------------ quadrature
// Gauss-Legendre nodes/weights on [-1,1] (roots of P_n by Newton iteration,
// w = 2/((1-x^2) P_n'(x)^2)), ascending order.  The reference takes its nodes
// from GSL's gsl_integration_glfixed with 2p+2 points per knot interval
// (functions/basis_bsplines.h:110, 375-414).
static void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w)
{
	x.assign(n, 0.0); w.assign(n, 0.0);
	const long double pi = 3.141592653589793238462643383279502884L;
	for (int i = 0; i < n; ++i) {
		long double z = std::cos(pi * ((long double)i + 0.75L) / ((long double)n + 0.5L)), dp = 1;
		for (int it = 0; it < 100; ++it) {
			long double p0 = 1, p1 = z;
			for (int k = 2; k <= n; ++k) { long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k; p0 = p1; p1 = p2; }
			if (n == 1) p0 = 1;
			dp = n * (z * p1 - p0) / (z * z - 1);
			long double dz = p1 / dp; z -= dz;
			if (std::fabs(dz) < 1e-19L) break;
		}
		long double p0 = 1, p1 = z;
		for (int k = 2; k <= n; ++k) { long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k; p0 = p1; p1 = p2; }
		if (n == 1) p0 = 1;
		dp = n * (z * p1 - p0) / (z * z - 1);
		x[n - 1 - i] = (double)z;
		w[n - 1 - i] = (double)(2 / ((1 - z * z) * dp * dp));
	}
}

// ------------------------------------------------------------------ B-splines
// Values and first derivatives of the p+1 B-splines of degree p that are
// non-zero on knot interval [t_s, t_{s+1}) at point x, by the Cox-de Boor
// triangular recursion.  out0[j], out1[j] belong to absolute spline s-p+j.
void bspline_eval(const std::vector<double>& t, int s, int p, double x, double* out0, double* out1)
{
	std::vector<double> N(p + 1, 0.0), left(p + 1), right(p + 1), Nm1(p + 1, 0.0);
	N[0] = 1.0;
	for (int q = 1; q <= p; ++q) {
		left[q] = x - t[s + 1 - q];
		right[q] = t[s + q] - x;
		if (q == p) Nm1 = N;	// degree p-1 values, for the derivative
		double saved = 0.0;
		for (int r = 0; r < q; ++r) {
			double den = right[r + 1] + left[q - r];
			double tmp = den == 0.0 ? 0.0 : N[r] / den;
			N[r] = saved + right[r + 1] * tmp;
			saved = left[q - r] * tmp;
		}
		N[q] = saved;
	}
	if (p == 0) Nm1[0] = 0.0;
	for (int j = 0; j <= p; ++j) out0[j] = N[j];
	// d/dx B_{i,p} = p [ B_{i,p-1}/(t_{i+p}-t_i) - B_{i+1,p-1}/(t_{i+p+1}-t_{i+1}) ]
	// Degree p-1 splines non-zero here: absolute s-p+1 .. s, stored in Nm1[0..p-1].
	for (int j = 0; j <= p; ++j) {
		int i = s - p + j;
		double a = 0.0, b = 0.0;
		if (j >= 1) { double d = t[i + p] - t[i]; a = d == 0.0 ? 0.0 : Nm1[j - 1] / d; }
		if (j <= p - 1) { double d = t[i + p + 1] - t[i + 1]; b = d == 0.0 ? 0.0 : Nm1[j] / d; }
		out1[j] = p * (a - b);
	}
}

// Knot vector of the reference's initialize_axis_linear_step
// (functions/basis_bsplines.h:450-459): p+1 copies of rmin, uniform interior
// step (rmax-rmin)/(n+2-p), p+1 copies of rmax; spline 0 and spline n+1 (the
// ones non-zero at the two end points) are dropped, leaving n active splines.
static std::vector<double> linear_knots(int n, int p, double rmin, double rmax)
{
	std::vector<double> t(n + p + 3);
	double step = (rmax - rmin) / (n + 2 - p);
	for (int i = 0; i < n + p + 3; ++i) {
		if (i < p) t[i] = rmin;
		else if (i < n + 2) t[i] = rmin + (i - p) * step;
		else t[i] = rmax;
	}
	return t;
}

void build_basis(radial_basis& B)
{
	int ni = B.nint();
	B.xq.assign((size_t)ni * B.nq, 0.0); B.wq.assign((size_t)ni * B.nq, 0.0);
	B.b0.assign((size_t)ni * (B.p + 1) * B.nq, 0.0); B.b1.assign((size_t)ni * (B.p + 1) * B.nq, 0.0);
	std::vector<double> gx, gw; gauss_legendre(B.nq, gx, gw);
	std::vector<double> v0(B.p + 1), v1(B.p + 1);
	for (int s = B.p; s < ni - B.p; ++s) {	// intervals [t_s, t_{s+1}), s in [p, n+2)
		double xl = B.t[s], xr = B.t[s + 1];
		if (xl == xr) continue;
		long double A = 0.5L * ((long double)xr + xl), H = 0.5L * ((long double)xr - xl);
		for (int k = 0; k < B.nq; ++k) {
			double x = (double)(A + H * gx[k]);
			B.xq[(size_t)s * B.nq + k] = x;
			B.wq[(size_t)s * B.nq + k] = (double)(H * gw[k]);
			bspline_eval(B.t, s, B.p, x, v0.data(), v1.data());
			for (int j = 0; j <= B.p; ++j) {
				B.b0[((size_t)s * (B.p + 1) + j) * B.nq + k] = v0[j];
				B.b1[((size_t)s * (B.p + 1) + j) * B.nq + k] = v1[j];
			}
		}
	}
}

// <d^mi B_i | f | d^mj B_j> over the active splines i, j (absolute i+1, j+1),
// summed interval by interval, node by node, as bsplines::integrate does
// (functions/basis_bsplines.h:262-289).
template <class F>
static double integrate(const radial_basis& B, int mi, int mj, int i, int j, const F& f)
{
	int ai = i + 1, aj = j + 1;
	int smin = std::max(ai, aj), smax = std::min(ai, aj) + B.p;
	double acc = 0.0;
	const auto& L = mi ? B.b1 : B.b0;
	const auto& R = mj ? B.b1 : B.b0;
	for (int s = smin; s <= smax; ++s) {
		if (s < B.p || s >= B.nint() - B.p) continue;
		int ji = ai - (s - B.p), jj = aj - (s - B.p);
		for (int k = 0; k < B.nq; ++k) {
			double x = B.xq[(size_t)s * B.nq + k];
			acc += B.wq[(size_t)s * B.nq + k] * f(x) * L[((size_t)s * (B.p + 1) + ji) * B.nq + k] * R[((size_t)s * (B.p + 1) + jj) * B.nq + k];
		}
	}
	return acc;
}

static double potential(const qpc_potential& v, double r)
{
	switch (v.kind) {
	case QPC_POTENTIAL_HYDROGENIC: return -v.zc / (r + 1e-50);
	case QPC_POTENTIAL_YUKAWA: return -(v.zc + v.zs * std::exp(-v.sigma * r)) / (r + 1e-50);
	default: return 0.0;
	}
}

// D^H Z_c D (real symmetric, N x N row-major) for coupling component comp of
// propagator_cn_hc_vgwr, with D = diag(phi_m), phi_m = 1 (mult 1) or i^(m - m0) (mult -i):
// Z(j, i) = mult * sgn * e(m, l) for j = (m+1, l+-1), e = outer (l+1) or inner (l-1)
// elements of Y11 (integrate_sinexp1/2) or Q11 (integrate_coslm1/2, sgn = -1 from
// operator_q11<dims_t,-1>::solve_eigen), basisfunc.hpp:243-299, operators/1e.hpp:336-523.
// The phase turns mult = -i into a factor conj(phi_{m+1}) (-i) phi_m = -1.
void vgwr_real_coupling(int n_l, int n_m, int m0, int comp, double* Zr)
{
	const int N = n_l * n_m;
	const bool q11 = comp == 1 || comp == 3;
	const bool imag = comp == 1 || comp == 2;
	auto outer = [&](long m, long l) {
		return q11 ? -std::sqrt(double((l + m + 1) * (l + m + 2)) / double((2 * l + 1) * (2 * l + 3))) * (l + 1)
			: -std::sqrt(double((l + m + 2) * (l + m + 1)) / double((2 * l + 1) * (2 * l + 3)));
	};
	auto inner = [&](long m, long l) {
		return q11 ? -std::sqrt(double((l - m) * (l - m - 1)) / double((2 * l + 1) * (2 * l - 1))) * l
			: +std::sqrt(double((l - m) * (l - m - 1)) / double((2 * l + 1) * (2 * l - 1)));
	};
	const double fac = (q11 ? -1.0 : 1.0) * (imag ? -1.0 : 1.0);
	for (size_t i = 0; i < (size_t)N * N; ++i) Zr[i] = 0.0;
	for (int im = 0; im + 1 < n_m; ++im)
		for (int il = 0; il < n_l; ++il) {
			long m = m0 + im, l = il + std::labs(m);
			long m2 = m + 1;
			for (int sgn = -1; sgn <= 1; sgn += 2) {
				long l2 = l + sgn;
				long il2 = l2 - std::labs(m2);
				if (l2 < 0 || il2 < 0 || il2 >= n_l) continue;
				double v = fac * (sgn > 0 ? outer(m, l) : inner(m, l));
				int i = im * n_l + il, j = (im + 1) * n_l + (int)il2;
				Zr[(size_t)j * N + i] = v;
				Zr[(size_t)i * N + j] = v;
			}
		}
}

} // namespace qpc

using namespace qpc;

extern "C" {

int qpc_linear_knots(int32_t n_r, int32_t p, double rmin, double rmax, double* knots)
{
	if (!knots || n_r < 2 * p + 2 || p < 1 || !(rmax > rmin)) return QPC_ERR_ARGS;
	auto t = linear_knots(n_r, p, rmin, rmax);
	std::memcpy(knots, t.data(), sizeof(double) * t.size());
	return QPC_OK;
}

int qpc_radial_setup(int32_t n_r, int32_t p, int32_t n_lh, const double* knots, const qpc_potential* pot, double mass,
	double* S, double* R, double* Rinv, double* D, double* H)
{
	if (n_r < 2 * p + 2 || p < 1 || p > QPC_MAX_RANK || n_lh < 0 || !knots || !(mass > 0)) return QPC_ERR_ARGS;
	if (H && (!pot || n_lh < 1)) return QPC_ERR_ARGS;
	radial_basis B;
	B.n = n_r; B.p = p; B.nq = 2 * p + 2;
	B.t.assign(knots, knots + n_r + p + 3);
	for (size_t i = 1; i < B.t.size(); ++i) if (B.t[i] < B.t[i - 1]) return QPC_ERR_ARGS;
	build_basis(B);
	const int ne = p + 1;
	const double coef = 0.5 / mass;
	for (int i = 0; i < n_r; ++i)
		for (int k = 0; k < ne; ++k) {
			int j = i + k;
			size_t o = (size_t)i * ne + k;
			bool in = j < n_r;
			if (S) S[o] = in ? integrate(B, 0, 0, i, j, [](double) { return 1.0; }) : 0.0;
			if (R) R[o] = in ? integrate(B, 0, 0, i, j, [](double r) { return r; }) : 0.0;
			if (Rinv) Rinv[o] = in ? integrate(B, 0, 0, i, j, [](double r) { return 1. / (r + 1e-50); }) : 0.0;
			if (D) D[o] = in ? integrate(B, 0, 1, i, j, [](double) { return 1.0; }) : 0.0;
		}
	if (H) {
		std::vector<double> vint((size_t)n_r * ne), kin((size_t)n_r * ne);
		for (int i = 0; i < n_r; ++i)
			for (int k = 0; k < ne && i + k < n_r; ++k) {
				vint[(size_t)i * ne + k] = integrate(B, 0, 0, i, i + k, [&](double r) { return potential(*pot, r); });
				kin[(size_t)i * ne + k] = integrate(B, 1, 1, i, i + k, [](double) { return 1.0; });
			}
		// H_l = <B|V|B> + <B|l(l+1)/r^2|B>/(2m) + <B'|B'>/(2m)  (spherical/utilities/basisfunc.hpp:93-106)
		for (int l = 0; l < n_lh; ++l) {
			double ll = (double)l * (l + 1);
			for (int i = 0; i < n_r; ++i)
				for (int k = 0; k < ne; ++k) {
					size_t o = (size_t)l * n_r * ne + (size_t)i * ne + k;
					if (i + k >= n_r) { H[o] = 0.0; continue; }
					double cent = integrate(B, 0, 0, i, i + k, [&](double r) { return ll / (r * r + 1e-50); });
					H[o] = vint[(size_t)i * ne + k] + cent * coef + kin[(size_t)i * ne + k] * coef;
				}
		}
	}
	return QPC_OK;
}

// <l,m|cos(theta)|l+1,m> = sqrt(((l+1)^2-m^2)/((2l+1)(2l+3)))  (spherical/utilities/basisfunc.hpp:222-229)
int qpc_y10_coupling(int32_t n_l, int32_t m, double* y10)
{
	if (n_l < 1 || !y10) return QPC_ERR_ARGS;
	long am = m < 0 ? -m : m;
	for (int il = 0; il < n_l; ++il) {
		long l = il + am;
		y10[il] = std::sqrt(double((l + 1) * (l + 1) - (long)m * m) / double((2 * l + 1) * (2 * l + 3)));
	}
	return QPC_OK;
}

// Eigen-decomposition of the symmetric tridiagonal Y10 block of one m (zero
// diagonal, off-diagonal y10(m, il)), the operator_y10::solve_eigen step of the
// reference (spherical/operators/1e.hpp:304-333).  lam ascending; P row-major,
// row a = eigenvector a.  Because the diagonal is zero, D Y D = -Y with
// D = diag((-1)^il): the eigenvalues come in pairs +-s and the eigenvector of -s
// is D times that of +s.  The vectors of the negative half are built that way
// exactly, and a zero eigenvalue (odd n_l) gets exactly zero odd components,
// which is what lets the engine transform with half the work.
// Method: cyclic Jacobi rotations on the dense matrix (Golub & Van Loan 8.5).
int qpc_y10_eigen(int32_t n_l, int32_t m, double* lam, double* P)
{
	if (n_l < 1 || !lam || !P) return QPC_ERR_ARGS;
	const int L = n_l;
	std::vector<double> y(L), A((size_t)L * L, 0.0), V((size_t)L * L, 0.0);
	qpc_y10_coupling(L, m, y.data());
	for (int i = 0; i + 1 < L; ++i) { A[(size_t)i * L + i + 1] = y[i]; A[(size_t)(i + 1) * L + i] = y[i]; }
	for (int i = 0; i < L; ++i) V[(size_t)i * L + i] = 1.0;
	for (int sweep = 0; sweep < 100; ++sweep) {
		double off = 0.0;
		for (int i = 0; i < L; ++i) for (int j = i + 1; j < L; ++j) off += A[(size_t)i * L + j] * A[(size_t)i * L + j];
		if (off < 1e-300) break;
		for (int pp = 0; pp < L; ++pp)
			for (int q = pp + 1; q < L; ++q) {
				double apq = A[(size_t)pp * L + q];
				if (std::fabs(apq) < 1e-300) continue;
				double app = A[(size_t)pp * L + pp], aqq = A[(size_t)q * L + q];
				double theta = (aqq - app) / (2 * apq);
				double tt = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
				double c = 1 / std::sqrt(tt * tt + 1), s = tt * c;
				for (int k = 0; k < L; ++k) {
					double akp = A[(size_t)k * L + pp], akq = A[(size_t)k * L + q];
					A[(size_t)k * L + pp] = c * akp - s * akq;
					A[(size_t)k * L + q] = s * akp + c * akq;
				}
				for (int k = 0; k < L; ++k) {
					double apk = A[(size_t)pp * L + k], aqk = A[(size_t)q * L + k];
					A[(size_t)pp * L + k] = c * apk - s * aqk;
					A[(size_t)q * L + k] = s * apk + c * aqk;
				}
				for (int k = 0; k < L; ++k) {
					double vkp = V[(size_t)k * L + pp], vkq = V[(size_t)k * L + q];
					V[(size_t)k * L + pp] = c * vkp - s * vkq;
					V[(size_t)k * L + q] = s * vkp + c * vkq;
				}
			}
	}
	std::vector<int> idx(L);
	for (int i = 0; i < L; ++i) idx[i] = i;
	std::sort(idx.begin(), idx.end(), [&](int a, int b) { return A[(size_t)a * L + a] < A[(size_t)b * L + b]; });
	const int npair = L / 2;
	// positive half: eigen-slot L-1-k holds +s_k (k = 0..npair-1), slot k holds -s_k
	for (int k = 0; k < npair; ++k) {
		int src = idx[L - 1 - k];
		double s = A[(size_t)src * L + src];
		double* vp = P + (size_t)(L - 1 - k) * L;
		double* vm = P + (size_t)k * L;
		// sign convention: first component positive
		double sg = V[(size_t)0 * L + src] >= 0 ? 1.0 : -1.0;
		for (int l = 0; l < L; ++l) { vp[l] = sg * V[(size_t)l * L + src]; vm[l] = (l & 1) ? -vp[l] : vp[l]; }
		lam[L - 1 - k] = s;
		lam[k] = -s;
	}
	if (L & 1) {
		int src = idx[npair];
		double* v0 = P + (size_t)npair * L;
		double nrm = 0.0, sg = V[(size_t)0 * L + src] >= 0 ? 1.0 : -1.0;
		for (int l = 0; l < L; ++l) { v0[l] = (l & 1) ? 0.0 : sg * V[(size_t)l * L + src]; nrm += v0[l] * v0[l]; }
		nrm = 1.0 / std::sqrt(nrm);
		for (int l = 0; l < L; ++l) v0[l] *= nrm;
		lam[npair] = 0.0;
	}
	return QPC_OK;
}

// Complex-symmetric banded LDL^T without pivoting of lower = S + i*g*H, stored
// as the engine consumes it: Lrow[r*p + (k-1)] = L(r, r-k), k = 1..p (zero
// where r-k < 0) and Dinv[r] = 1/D(r), both complex (re, im).  This is the
// factorisation cn_component_hc::initialize obtains with lu_zsb
// (spherical/propagator/cn_1e.hpp:342-360, algorithm/ed.h:208-289); returns the
// number of pivots with |D|^2 < 1e-31, as lu_zsb counts them.
int qpc_ldlt_csym(int32_t n, int32_t p, const double* S, const double* H, double g, double* Lrow, double* Dinv)
{
	if (n < 2 * p + 2 || p < 1 || !S || !H || !Lrow || !Dinv) return -1;
	const int ne = p + 1;
	// window W[a][b] (b <= a), rows i..i+p, complex
	std::vector<double> wre((size_t)ne * ne, 0.0), wim((size_t)ne * ne, 0.0);
	auto band_re = [&](int r, int c) { int a = std::min(r, c), k = std::abs(r - c); return (k > p || std::max(r, c) >= n) ? 0.0 : S[(size_t)a * ne + k]; };
	auto band_im = [&](int r, int c) { int a = std::min(r, c), k = std::abs(r - c); return (k > p || std::max(r, c) >= n) ? 0.0 : g * H[(size_t)a * ne + k]; };
	for (int a = 0; a < ne; ++a)
		for (int b = 0; b <= a; ++b) { wre[a * ne + b] = band_re(a, b); wim[a * ne + b] = band_im(a, b); }
	std::vector<double> col_re((size_t)n * ne, 0.0), col_im((size_t)n * ne, 0.0);
	int bad = 0;
	for (int i = 0; i < n; ++i) {
		double dr = wre[0], di = wim[0];
		double den = dr * dr + di * di;
		if (den < 1e-31) bad++;
		double rr = dr / den, ri = -di / den;
		Dinv[2 * (size_t)i] = rr; Dinv[2 * (size_t)i + 1] = ri;
		double lre[QPC_MAX_RANK + 1], lim[QPC_MAX_RANK + 1];
		for (int a = 1; a < ne; ++a) {
			double xr = wre[a * ne], xi = wim[a * ne];
			lre[a] = xr * rr - xi * ri; lim[a] = xr * ri + xi * rr;
			col_re[(size_t)i * ne + a] = lre[a]; col_im[(size_t)i * ne + a] = lim[a];
		}
		// trailing update and shift: W'[a-1][b-1] = W[a][b] - l_a * W[b][0]
		std::vector<double> nre((size_t)ne * ne, 0.0), nim((size_t)ne * ne, 0.0);
		for (int a = 1; a < ne; ++a)
			for (int b = 1; b <= a; ++b) {
				double xr = wre[b * ne], xi = wim[b * ne];
				nre[(a - 1) * ne + b - 1] = wre[a * ne + b] - (lre[a] * xr - lim[a] * xi);
				nim[(a - 1) * ne + b - 1] = wim[a * ne + b] - (lre[a] * xi + lim[a] * xr);
			}
		int rnew = i + ne;
		for (int b = 0; b < ne; ++b) { nre[p * ne + b] = band_re(rnew, i + 1 + b); nim[p * ne + b] = band_im(rnew, i + 1 + b); }
		wre.swap(nre); wim.swap(nim);
	}
	for (int r = 0; r < n; ++r)
		for (int k = 1; k <= p; ++k) {
			size_t o = 2 * ((size_t)r * p + (k - 1));
			if (r - k < 0) { Lrow[o] = 0.0; Lrow[o + 1] = 0.0; continue; }
			Lrow[o] = col_re[(size_t)(r - k) * ne + k];
			Lrow[o + 1] = col_im[(size_t)(r - k) * ne + k];
		}
	return bad;
}

// banded Cholesky S = G G^T, G lower, row form G[i][i-k] at g[i*(p+1)+k] (right-hand
// loop over the band, the column-by-column algorithm of Golub & Van Loan 4.3.5);
// returns 0, or 1 + the row of the first non-positive pivot
static int chol_band_rows(int n, int p, const double* S, double* g)
{
	const int ne = p + 1;
	for (size_t i = 0; i < (size_t)n * ne; ++i) g[i] = 0.0;
	for (int i = 0; i < n; ++i) {
		for (int k = p; k >= 0; --k) {
			int j = i - k;
			if (j < 0) continue;
			double s = S[(size_t)j * ne + k];	// S(j, i)
			for (int q = 1; q <= p; ++q) {
				int c = j - q;	// column c < j, need G[i][c], G[j][c]
				if (c < 0 || i - c > p) continue;
				s -= g[(size_t)i * ne + (i - c)] * g[(size_t)j * ne + (j - c)];
			}
			if (k == 0) {
				if (!(s > 0)) return i + 1;
				g[(size_t)i * ne] = std::sqrt(s);
			} else g[(size_t)i * ne + k] = s / g[(size_t)j * ne];
		}
	}
	return 0;
}

// Eigen-decomposition of a dense real symmetric matrix a (n x n, row-major, both
// triangles): Householder tridiagonalisation and implicit QL with Wilkinson shifts
// (Golub & Van Loan 8.3).  On return d holds the eigenvalues (unsorted) and column i
// of a the eigenvector of d[i].  Returns QPC_OK or QPC_ERR_NUMERIC.
static int sym_eigen(int n, std::vector<double>& a, std::vector<double>& d)
{
	d.assign(n, 0.0);
	std::vector<double> e(n);
	// Householder tridiagonalisation, accumulating Q in C (rows of Q^T)
	for (int i = n - 1; i > 0; --i) {
		int l = i - 1;
		double h = 0.0, scale = 0.0;
		if (l > 0) {
			for (int k = 0; k <= l; ++k) scale += std::fabs(a[(size_t)i * n + k]);
			if (scale == 0.0) e[i] = a[(size_t)i * n + l];
			else {
				for (int k = 0; k <= l; ++k) { a[(size_t)i * n + k] /= scale; h += a[(size_t)i * n + k] * a[(size_t)i * n + k]; }
				double f = a[(size_t)i * n + l];
				double gg = f >= 0 ? -std::sqrt(h) : std::sqrt(h);
				e[i] = scale * gg; h -= f * gg; a[(size_t)i * n + l] = f - gg; f = 0.0;
				for (int j = 0; j <= l; ++j) {
					a[(size_t)j * n + i] = a[(size_t)i * n + j] / h;
					double s = 0.0;
					for (int k = 0; k <= j; ++k) s += a[(size_t)j * n + k] * a[(size_t)i * n + k];
					for (int k = j + 1; k <= l; ++k) s += a[(size_t)k * n + j] * a[(size_t)i * n + k];
					e[j] = s / h; f += e[j] * a[(size_t)i * n + j];
				}
				double hh = f / (h + h);
				for (int j = 0; j <= l; ++j) {
					double ff = a[(size_t)i * n + j];
					e[j] = gg = e[j] - hh * ff;
					for (int k = 0; k <= j; ++k) a[(size_t)j * n + k] -= (ff * e[k] + gg * a[(size_t)i * n + k]);
				}
			}
		} else e[i] = a[(size_t)i * n + l];
		d[i] = h;
	}
	d[0] = 0.0; e[0] = 0.0;
	for (int i = 0; i < n; ++i) {
		int l = i - 1;
		if (d[i] != 0.0) {
			for (int j = 0; j <= l; ++j) {
				double s = 0.0;
				for (int k = 0; k <= l; ++k) s += a[(size_t)i * n + k] * a[(size_t)k * n + j];
				for (int k = 0; k <= l; ++k) a[(size_t)k * n + j] -= s * a[(size_t)k * n + i];
			}
		}
		d[i] = a[(size_t)i * n + i];
		a[(size_t)i * n + i] = 1.0;
		for (int j = 0; j <= l; ++j) { a[(size_t)j * n + i] = 0.0; a[(size_t)i * n + j] = 0.0; }
	}
	// implicit QL
	for (int i = 1; i < n; ++i) e[i - 1] = e[i];
	e[n - 1] = 0.0;
	for (int l = 0; l < n; ++l) {
		int iter = 0, m;
		do {
			for (m = l; m < n - 1; ++m) {
				double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
				if (std::fabs(e[m]) <= 1e-16 * dd) break;
			}
			if (m != l) {
				if (iter++ == 60) return QPC_ERR_NUMERIC;
				double gg = (d[l + 1] - d[l]) / (2.0 * e[l]);
				double r = std::hypot(gg, 1.0);
				gg = d[m] - d[l] + e[l] / (gg + (gg >= 0 ? std::fabs(r) : -std::fabs(r)));
				double s = 1.0, c = 1.0, pp = 0.0;
				int i;
				for (i = m - 1; i >= l; --i) {
					double f = s * e[i], b = c * e[i];
					e[i + 1] = (r = std::hypot(f, gg));
					if (r == 0.0) { d[i + 1] -= pp; e[m] = 0.0; break; }
					s = f / r; c = gg / r; gg = d[i + 1] - pp; r = (d[i] - gg) * s + 2.0 * c * b; d[i + 1] = gg + (pp = s * r); gg = c * r - b;
					for (int k = 0; k < n; ++k) {
						f = a[(size_t)k * n + i + 1];
						a[(size_t)k * n + i + 1] = s * a[(size_t)k * n + i] + c * f;
						a[(size_t)k * n + i] = c * a[(size_t)k * n + i] - s * f;
					}
				}
				if (r == 0.0 && i >= l) continue;
				d[l] -= pp; e[l] = gg; e[m] = 0.0;
			}
		} while (m != l);
	}
	return QPC_OK;
}

// Eigenpairs of the generalized banded problem H v = E S v for one l block,
// the gv_dsb (LAPACKE_dsbgv) call of the reference (algorithm/ed.h:105-112,
// used by coefficient::initialize, spherical/coefficient/1e.hpp:91-143, and
// eigenstate_sph::initialize, spherical/spectrum/population_1e.hpp:58-118).
// Eigenvalues ascending; vec row j = eigenvector j, S-normalised.
// Method: Cholesky S = G G^T (banded), C = G^-1 H G^-T (dense), Householder
// tridiagonalisation and implicit QL with Wilkinson shifts (Golub & Van Loan
// 8.3), back-transformed by G^-T.  n_want <= n: only the lowest n_want vectors
// are written (all eigenvalues are).
int qpc_gen_eigen(int32_t n, int32_t p, const double* S, const double* Hl, int32_t n_want, double* energy, double* vec)
{
	if (n < 2 * p + 2 || p < 1 || !S || !Hl || !energy || n_want < 0 || n_want > n || (n_want && !vec)) return QPC_ERR_ARGS;
	const int ne = p + 1;
	// banded Cholesky, G lower: G[i][i-k] stored g[i*ne+k]
	std::vector<double> g((size_t)n * ne, 0.0);
	if (chol_band_rows(n, p, S, g.data())) return QPC_ERR_SINGULAR;
	// C = G^-1 H G^-T : first X = G^-1 H (dense n x n), then C = G^-1 X^T
	std::vector<double> X((size_t)n * n, 0.0), C((size_t)n * n, 0.0);
	auto hval = [&](int r, int c) { int a = std::min(r, c), k = std::abs(r - c); return k > p ? 0.0 : Hl[(size_t)a * ne + k]; };
	for (int col = 0; col < n; ++col) {
		for (int i = 0; i < n; ++i) {
			double s = hval(i, col);
			for (int k = 1; k <= p && i - k >= 0; ++k) s -= g[(size_t)i * ne + k] * X[(size_t)(i - k) * n + col];
			X[(size_t)i * n + col] = s / g[(size_t)i * ne];
		}
	}
	for (int col = 0; col < n; ++col) {
		for (int i = 0; i < n; ++i) {
			double s = X[(size_t)col * n + i];
			for (int k = 1; k <= p && i - k >= 0; ++k) s -= g[(size_t)i * ne + k] * C[(size_t)(i - k) * n + col];
			C[(size_t)i * n + col] = s / g[(size_t)i * ne];
		}
	}
	for (int i = 0; i < n; ++i) for (int j = 0; j < i; ++j) { double m = 0.5 * (C[(size_t)i * n + j] + C[(size_t)j * n + i]); C[(size_t)i * n + j] = m; C[(size_t)j * n + i] = m; }
	std::vector<double> d;
	if (int rc = sym_eigen(n, C, d)) return rc;
	std::vector<double>& a = C;
	std::vector<int> idx(n);
	for (int i = 0; i < n; ++i) idx[i] = i;
	std::sort(idx.begin(), idx.end(), [&](int x, int y) { return d[x] < d[y]; });
	for (int j = 0; j < n; ++j) energy[j] = d[idx[j]];
	// eigenvector of the pencil: v = G^-T y, with y = column idx[j] of a
	for (int j = 0; j < n_want; ++j) {
		double* v = vec + (size_t)j * n;
		for (int i = 0; i < n; ++i) v[i] = a[(size_t)i * n + idx[j]];
		for (int i = n - 1; i >= 0; --i) {
			double s = v[i];
			for (int k = 1; k <= p && i + k < n; ++k) s -= g[(size_t)(i + k) * ne + k] * v[i + k];
			v[i] = s / g[(size_t)i * ne];
		}
	}
	return QPC_OK;
}

// absorber_mask::initialize (absorber.hpp:42-49): M = <B_i| m(r) |B_j> with m(r) = 1 for
// r < rmin, 0 for r > rmax, |cos(pi/2 (r - rmin)/(rmax - rmin))|^index between, by the same
// quadrature as the other radial matrices (integrate_0r0).
int qpc_mask_band(int32_t n_r, int32_t p, const double* knots, double rmin, double rmax, double index, double* M)
{
	if (n_r < 2 * p + 2 || p < 1 || p > QPC_MAX_RANK || !knots || !M || !(rmax > rmin)) return QPC_ERR_ARGS;
	radial_basis B;
	B.n = n_r; B.p = p; B.nq = 2 * p + 2;
	B.t.assign(knots, knots + n_r + p + 3);
	for (size_t i = 1; i < B.t.size(); ++i) if (B.t[i] < B.t[i - 1]) return QPC_ERR_ARGS;
	build_basis(B);
	const double pi = 3.14159265358979323846;
	auto f = [&](double r) { return r < rmin ? 1.0 : r > rmax ? 0.0 : std::pow(std::fabs(std::cos(0.5 * pi * (r - rmin) / (rmax - rmin))), index); };
	const int ne = p + 1;
	for (int i = 0; i < n_r; ++i)
		for (int k = 0; k < ne; ++k) M[(size_t)i * ne + k] = i + k < n_r ? integrate(B, 0, 0, i, i + k, f) : 0.0;
	return QPC_OK;
}

// lu_dsb (LAPACKE_dpbtrf 'L', algorithm/ed.h:182-193) in operator_sc's layout
// (operators/1e.hpp:1233-1244): L(r+k, r) at L[r*(p+1)+k], zero past the last row
int qpc_cholesky_band(int32_t n, int32_t p, const double* S, double* L)
{
	if (n < 1 || p < 0 || !S || !L) return -1;
	const int ne = p + 1;
	std::vector<double> g((size_t)n * ne);
	int bad = chol_band_rows(n, p, S, g.data());
	if (bad) return bad;
	for (int r = 0; r < n; ++r)
		for (int k = 0; k <= p; ++k) L[(size_t)r * ne + k] = r + k < n ? g[(size_t)(r + k) * ne + k] : 0.0;
	return 0;
}

// Angular couplings of the velocity-gauge elliptical propagator propagator_cn_hc_vgwr
// (cn_1e.hpp:836-890) on the channels ch = im*n_l + il (m = m0 + im, l = |m| + il):
//   comp 0 (x1): Y11 (sin e^{-i phi}, integrate_sinexp1/2), mult 1
//   comp 1 (x2): Q11 (-cos L_- - sin e^{-i phi}(1 - L_z), integrate_coslm1/2, sign -1), mult -i
//   comp 2 (y1): Y11, mult -i
//   comp 3 (y2): Q11, mult 1
// (basisfunc.hpp:243-299, operators/1e.hpp:336-523).  Z(j, i) = mult * outer(m, l) for
// j = (m+1, l+1) and mult * inner(m, l) for j = (m+1, l-1) when j is on the grid, Z(i, j)
// = conj Z(j, i).  Output: lam[k] ascending and P[k][ch] complex (rows = conjugated
// eigenvectors, P Z P^H = diag(lam)), the transform construct applies
// (cn_transform_hm, cn_1e.hpp:151-293, after solve_eigen and conjugate()).
// Method: Z couples m only to m +- 1 and keeps il mod 2, and D^H Z D is real symmetric
// for D = diag(phi_m), phi_m = 1 (mult 1) or i^(m - m0) (mult -i); each il-parity block
// of the real matrix is diagonalised by sym_eigen.  Eigenvectors of degenerate
// eigenvalues differ from LAPACK's; the propagator depends only on the spectral
// projectors.
int qpc_vgwr_angular(int32_t n_l, int32_t n_m, int32_t m0, int32_t comp, double* lam, double* P)
{
	if (n_l < 1 || n_m < 1 || comp < 0 || comp > 3 || !lam || !P) return QPC_ERR_ARGS;
	const int N = n_l * n_m;
	const bool imag = comp == 1 || comp == 2;	// mult = -i
	std::vector<double> Zr((size_t)N * N, 0.0);
	vgwr_real_coupling(n_l, n_m, m0, comp, Zr.data());
	// eigenvectors block by block (il parity)
	std::vector<double> evals;
	std::vector<std::vector<double>> evecs;	// full-length real vectors
	for (int par = 0; par < 2; ++par) {
		std::vector<int> idx;
		for (int ch = 0; ch < N; ++ch) if ((ch % n_l) % 2 == par) idx.push_back(ch);
		const int nb = (int)idx.size();
		if (!nb) continue;
		std::vector<double> a((size_t)nb * nb), d;
		for (int r = 0; r < nb; ++r)
			for (int c = 0; c < nb; ++c) a[(size_t)r * nb + c] = Zr[(size_t)idx[r] * N + idx[c]];
		if (int rc = sym_eigen(nb, a, d)) return rc;
		for (int k = 0; k < nb; ++k) {
			std::vector<double> v(N, 0.0);
			for (int r = 0; r < nb; ++r) v[idx[r]] = a[(size_t)r * nb + k];
			evals.push_back(d[k]);
			evecs.push_back(std::move(v));
		}
	}
	std::vector<int> ord(N);
	for (int k = 0; k < N; ++k) ord[k] = k;
	std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return evals[x] < evals[y]; });
	for (int k = 0; k < N; ++k) {
		lam[k] = evals[ord[k]];
		const std::vector<double>& v = evecs[ord[k]];
		for (int ch = 0; ch < N; ++ch) {
			// P[k][ch] = conj(phi_m) v[ch], phi_m = i^(im) when mult = -i
			int im = ch / n_l, r4 = imag ? im & 3 : 0;
			double re = 0.0, imv = 0.0;
			switch (r4) {	// conj(i^r4) = (-i)^r4
			case 0: re = v[ch]; break;
			case 1: imv = -v[ch]; break;
			case 2: re = -v[ch]; break;
			default: imv = v[ch]; break;
			}
			P[2 * ((size_t)k * N + ch)] = re;
			P[2 * ((size_t)k * N + ch) + 1] = imv;
		}
	}
	return QPC_OK;
}

// E(t) of one field_component_sinen<n> (structure/field.h:89-133):
// E0 sin^n(pi (t-t0)/tau) sin(w t + cep) on (t0, t0+tau), tau = nc 2pi/w,
// t0 = n0 2pi/w, cep given in units of pi.  The time grid is the reference's
// field<>: t_i = t_min + i dt, i = 0..nt with nt = 1 + floor((t_max-t_min)/dt)
// (structure/field.h:245-281).  Writes nt+1 values f[0..nt] when f != NULL and
// returns nt via *nt_out.
int qpc_field_sinen(int32_t n_pow, double e0, double w0, double nc, double n0, double cep, double dt, int64_t cap, double* f, int64_t* nt_out)
{
	if (!(w0 > 0) || !(dt > 0) || !(nc > 0) || n_pow < 0 || !nt_out) return QPC_ERR_ARGS;
	double pd = 6.283185307179586 / w0;
	double phi = 3.141592653589793 * cep;
	double tau = nc * pd, ini = n0 * pd;
	double tmin = ini, tmax = ini + tau;
	int64_t nt = (int64_t)(size_t)(1.0 + (tmax - tmin) / dt);
	*nt_out = nt;
	if (!f) return QPC_OK;
	if (cap < nt + 1) return QPC_ERR_ARGS;
	for (int64_t i = 0; i <= nt; ++i) {
		double t = tmin + dt * (double)i;
		double ts = (t - ini) / tau;
		double ev = (t > ini && t < ini + tau) ? std::pow(std::sin(3.1415926535897932 * ts), n_pow) : 0.0;
		double ca = e0 * std::sin(w0 * t + phi);
		f[i] = ca * ev;
	}
	return QPC_OK;
}

} // extern "C"
