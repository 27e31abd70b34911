// Stand-in for the GNU Scientific Library headers, used ONLY to compile the
// unmodified reference headers into the test oracle under oracle/_ref/.
//
// Test infrastructure, not product code.  The one GSL facility on the
// reference's time-stepping path is fixed-order Gauss-Legendre quadrature
// (gsl_integration_glfixed_*), used to build the B-spline matrices.  It is
// restated here from the textbook method: the n nodes are the roots of the
// Legendre polynomial P_n, found by Newton iteration from the Chebyshev-like
// initial guess cos(pi (i - 1/4) / (n + 1/2)), with weights
// w_i = 2 / ((1 - x_i^2) P_n'(x_i)^2); iteration is carried in long double.
// Points are returned in increasing order, as GSL documents for
// gsl_integration_glfixed_point.  The Legendre and trigonometric routines the
// momentum spectra use are restated below; everything else is declared only.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

struct gsl_integration_glfixed_table { size_t n; std::vector<long double> x, w; };

static inline gsl_integration_glfixed_table* gsl_integration_glfixed_table_alloc(size_t n)
{
	auto* t = new gsl_integration_glfixed_table; t->n = n; t->x.resize(n); t->w.resize(n);
	const long double pi = 3.141592653589793238462643383279502884L;
	for (size_t i = 0; i < n; ++i) {
		long double z = std::cos(pi * ((long double)i + 0.75L) / ((long double)n + 0.5L));
		long double dp = 0;
		for (int it = 0; it < 100; ++it) {
			long double p0 = 1, p1 = z;
			for (size_t k = 2; k <= n; ++k) { long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k; p0 = p1; p1 = p2; }
			long double pn = (n == 0) ? 1 : (n == 1 ? z : p1);
			if (n == 1) p0 = 1;
			dp = n * (z * pn - p0) / (z * z - 1);
			long double dz = pn / dp; z -= dz;
			if (std::fabs(dz) < 1e-19L) break;
		}
		{ long double p0 = 1, p1 = z;
		  for (size_t k = 2; k <= n; ++k) { long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k; p0 = p1; p1 = p2; }
		  dp = n * (z * p1 - p0) / (z * z - 1); }
		// roots come out in decreasing order of z; store ascending
		t->x[n - 1 - i] = z; t->w[n - 1 - i] = 2 / ((1 - z * z) * dp * dp);
	}
	return t;
}
static inline void gsl_integration_glfixed_table_free(gsl_integration_glfixed_table* t) { delete t; }
static inline int gsl_integration_glfixed_point(double a, double b, size_t i, double* xi, double* wi, const gsl_integration_glfixed_table* t)
{
	long double A = 0.5L * ((long double)b + a), B = 0.5L * ((long double)b - a);
	*xi = (double)(A + B * t->x[i]); *wi = (double)(B * t->w[i]); return 0;
}

[[noreturn]] static inline void qpc_gsl_shim_unsupported(const char* what)
{ std::fprintf(stderr, "oracle shim: GSL routine %s is not available in this harness\n", what); std::abort(); }
#define QPC_GSL_UNSUPPORTED(ret, name) template <class... A> static inline ret name(A...) { qpc_gsl_shim_unsupported(#name); }
typedef enum { GSL_SF_LEGENDRE_SCHMIDT, GSL_SF_LEGENDRE_SPHARM, GSL_SF_LEGENDRE_FULL, GSL_SF_LEGENDRE_NONE } gsl_sf_legendre_t;
struct gsl_sf_result { double val, err; };
// Trigonometric functions and the associated Legendre array routines of GSL's documented
// interface, for the momentum-spectrum classes (spectrum/momentum_1e.hpp): the array holds
// P_l^m(x) for 0 <= m <= l <= lmax at index l(l+1)/2 + m; GSL_SF_LEGENDRE_SPHARM scales it by
// sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!), csphase = -1 includes the Condon-Shortley phase (-1)^m.
// Computed by the textbook recurrences in m (diagonal) and l, in long double.
static inline double gsl_sf_cos(double x) { return std::cos(x); }
static inline double gsl_sf_sin(double x) { return std::sin(x); }
static inline size_t gsl_sf_legendre_array_index(size_t l, size_t m) { return l * (l + 1) / 2 + m; }
static inline size_t gsl_sf_legendre_array_n(size_t lmax) { return (lmax + 1) * (lmax + 2) / 2; }
static inline int gsl_sf_legendre_array_e(gsl_sf_legendre_t norm, size_t lmax, double x, double csphase, double* out)
{
	if (norm != GSL_SF_LEGENDRE_SPHARM) qpc_gsl_shim_unsupported("gsl_sf_legendre_array_e (normalisation other than SPHARM)");
	const long double pi = 3.141592653589793238462643383279502884L;
	const long double X = x, s = std::sqrt((1.0L - X) * (1.0L + X));
	long double ymm = std::sqrt(1.0L / (4.0L * pi));
	for (size_t m = 0; m <= lmax; ++m) {
		if (m > 0) ymm *= (csphase < 0 ? -1.0L : 1.0L) * s * std::sqrt((2.0L * m + 1.0L) / (2.0L * m));
		out[m * (m + 1) / 2 + m] = (double)ymm;
		if (m == lmax) break;
		long double y0 = ymm, y1 = X * std::sqrt(2.0L * m + 3.0L) * ymm;
		out[(m + 1) * (m + 2) / 2 + m] = (double)y1;
		for (size_t l = m + 2; l <= lmax; ++l) {
			const long double L = (long double)l, M = (long double)m;
			const long double a = std::sqrt((4.0L * L * L - 1.0L) / (L * L - M * M));
			const long double b = std::sqrt(((L - 1) * (L - 1) - M * M) / (4.0L * (L - 1) * (L - 1) - 1.0L));
			const long double y2 = a * (X * y1 - b * y0);
			out[l * (l + 1) / 2 + m] = (double)y2;
			y0 = y1; y1 = y2;
		}
	}
	return 0;
}
QPC_GSL_UNSUPPORTED(double, gsl_sf_coupling_3j)
QPC_GSL_UNSUPPORTED(int, gsl_sf_legendre_deriv1_alt_array_e)
QPC_GSL_UNSUPPORTED(int, gsl_sf_legendre_deriv1_array_e)
QPC_GSL_UNSUPPORTED(int, gsl_sf_legendre_deriv2_alt_array_e)
QPC_GSL_UNSUPPORTED(int, gsl_sf_legendre_deriv2_array_e)
