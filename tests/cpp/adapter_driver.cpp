// The C++ drop-in binding (include/qpc_gb300_lgwz.hpp) compiled against the reference's
// own headers: the reference's propagator_cn_hc_lgwz and the binding are initialised with
// the same integrator_radi / integrator_angu / potential / dt, as binsrc/sphTDSE.cpp:742-776
// does, and both advance the same coefficient<dims_t> through field steps
// (propagate(coef, f_ti, f_tf)) and field-free steps (propagate(coef)), as the driver loop
// of binsrc/sphTDSE.cpp:786-831 calls them.
//
// Test infrastructure (tests/test_adapter_build.py builds and runs it where the reference
// checkout exists).  Exit codes: 0 results agree (GPU present), 1 they differ, 3 the
// binding's initialize threw errn_t because no usable GPU is present (its error channel),
// 2 anything else.
#include <spherical/inventory.h>
#include "qpc_gb300_lgwz.hpp"
#include <cmath>
#include <cstdio>
#include <vector>

using namespace qpc;
using namespace qpc::spherical;

using dims_t = dimension_1e<64, 6, 6, 1, 0>;

static void fill(coefficient<dims_t>& c)
{
	// a smooth, deterministic state in every (l, r) channel, (re, im) interleaved
	double* d = c.dptr();
	for (size_t il = 0; il < dims_t::l_dims; ++il)
		for (size_t ir = 0; ir < dims_t::n_dims; ++ir) {
			const double r = (double)ir;
			const size_t i = il * dims_t::n_dims + ir;
			d[2 * i] = std::exp(-r / 9.0) * std::cos(0.3 * r + il);
			d[2 * i + 1] = std::exp(-r / 11.0) * std::sin(0.2 * r - il);
		}
}

int main()
{
	const double rmax = 30.0, dt = 0.05;
	auto radi = integrator_radi<dims_t>();
	auto angu = integrator_angu<dims_t>();
	radi.initialize(0.0, rmax);
	const hydrogenic potn{1.0};
	auto ref = propagator_cn_hc_lgwz<dims_t>();
	ref.initialize(1, radi, angu, 1.0, potn, dt);
	qpc_gb300::propagator_cn_hc_lgwz<dims_t> gpu;
	try {
		gpu.initialize(1, radi, angu, 1.0, potn, dt);
	} catch (const errn_t& e) {
		std::printf("binding initialize threw errn_t: ");
		std::fflush(stdout);
		e.what();	// the reference's errn_t prints its message (utilities/error.h)
		std::fflush(stdout);
		return 3;
	}
	coefficient<dims_t> a, b;
	fill(a);
	fill(b);
	const int nt = 25, nfree = 5;
	std::vector<double> f(nt + 1);
	for (int i = 0; i <= nt; ++i) f[i] = 0.05 * std::sin(0.2 * i);
	for (int i = 0; i < nt; ++i) {
		ref.propagate(a, f[i], f[i + 1]);
		gpu.propagate(b, f[i], f[i + 1]);
		if (gpu.last_status() != QPC_OK) { std::printf("binding propagate failed: %s\n", qpc_last_error()); return 2; }
	}
	for (int i = 0; i < nfree; ++i) {
		ref.propagate(a);
		gpu.propagate(b);
	}
	double num = 0.0, den = 0.0;
	const double *x = a.dptr(), *y = b.dptr();
	for (size_t i = 0; i < 2 * dims_t::n_leng; ++i) {
		num += (x[i] - y[i]) * (x[i] - y[i]);
		den += x[i] * x[i];
	}
	const double err = std::sqrt(num / den);
	std::printf("binding vs reference after %d field + %d field-free steps: rel L2 %.3e\n", nt, nfree, err);
	return err < 1e-12 ? 0 : 1;
}
