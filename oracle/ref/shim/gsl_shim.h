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
// gsl_integration_glfixed_point.  Everything else is declared only.
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
QPC_GSL_UNSUPPORTED(double, gsl_sf_cos)
QPC_GSL_UNSUPPORTED(double, gsl_sf_sin)
QPC_GSL_UNSUPPORTED(double, gsl_sf_coupling_3j)
QPC_GSL_UNSUPPORTED(int, gsl_sf_legendre_array_e)
QPC_GSL_UNSUPPORTED(size_t, gsl_sf_legendre_array_index)
QPC_GSL_UNSUPPORTED(size_t, gsl_sf_legendre_array_n)
QPC_GSL_UNSUPPORTED(int, gsl_sf_legendre_deriv1_alt_array_e)
QPC_GSL_UNSUPPORTED(int, gsl_sf_legendre_deriv1_array_e)
QPC_GSL_UNSUPPORTED(int, gsl_sf_legendre_deriv2_alt_array_e)
QPC_GSL_UNSUPPORTED(int, gsl_sf_legendre_deriv2_array_e)
