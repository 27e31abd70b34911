// The reference driver's length-gauge loop (binsrc/sphTDSE.cpp:742-831) written in C++ over the C ABI
// of include/qpc_gb300.h, with no Python in between: radial setup on the host (qpc_linear_knots,
// qpc_radial_setup; integrator_radi::initialize and the operators' initialize), the propagator
// (qpc_lgwz_create; propagator_cn_hc_lgwz::initialize), the state (qpc_lgwz_put / get; the
// coefficient<dims_t> layout), the step loop -- one qpc_lgwz_run for the whole pulse, or with
// "stepwise" one propagate(f_i, f_i+1) per field step and propagate() per field-free step, as the
// reference's loop calls its propagator -- and the S-norm (operator_rsym::observe).
//
// usage: lgwz_driver N P L RMAX DT INIT FIELD NT NFREE OUT [stepwise]
//   INIT  raw float64, the complex state c[l][r] (2 L N values); FIELD raw float64 f(t_0..t_NT)
//   OUT   raw float64: the final state (2 L N values) followed by its S-norm
// Test infrastructure for tests/test_gpu_cpp_driver.py.
#include "qpc_gb300.h"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

static std::vector<double> slurp(const char* path, size_t n)
{
	std::vector<double> v(n);
	FILE* f = std::fopen(path, "rb");
	if (!f || std::fread(v.data(), sizeof(double), n, f) != n) { std::fprintf(stderr, "cannot read %s\n", path); std::exit(2); }
	std::fclose(f);
	return v;
}

static void check(int rc, const char* what)
{
	if (rc != QPC_OK) { std::fprintf(stderr, "%s: status %d: %s\n", what, rc, qpc_last_error()); std::exit(1); }
}

int main(int argc, char** argv)
{
	if (argc < 11) { std::fprintf(stderr, "usage: lgwz_driver N P L RMAX DT INIT FIELD NT NFREE OUT [stepwise]\n"); return 2; }
	const int N = std::atoi(argv[1]), P = std::atoi(argv[2]), L = std::atoi(argv[3]);
	const double rmax = std::atof(argv[4]), dt = std::atof(argv[5]);
	const int64_t nt = std::atoll(argv[8]), nfree = std::atoll(argv[9]);
	const bool stepwise = argc > 11 && std::string(argv[11]) == "stepwise";
	const size_t NE = P + 1;
	std::vector<double> knots(N + P + 3), S(N * NE), R(N * NE), H((size_t)L * N * NE);
	check(qpc_linear_knots(N, P, 0.0, rmax, knots.data()), "qpc_linear_knots");
	qpc_potential pot{QPC_POTENTIAL_HYDROGENIC, 1.0, 0.0, 0.0};
	check(qpc_radial_setup(N, P, L, knots.data(), &pot, 1.0, S.data(), R.data(), nullptr, nullptr, H.data()), "qpc_radial_setup");
	qpc_dims d{N, P, L, 1, 0, 1};
	qpc_lgwz* prop = nullptr;
	check(qpc_lgwz_create(&d, dt, S.data(), R.data(), H.data(), &prop), "qpc_lgwz_create");
	std::vector<double> c = slurp(argv[6], 2 * (size_t)L * N), f = slurp(argv[7], nt + 1);
	check(qpc_lgwz_put(prop, c.data()), "qpc_lgwz_put");
	if (stepwise) {
		for (int64_t it = 0; it < nt + nfree; ++it) {
			if (it < nt) check(qpc_lgwz_propagate(prop, &f[it], &f[it + 1]), "qpc_lgwz_propagate");
			else check(qpc_lgwz_propagate_free(prop), "qpc_lgwz_propagate_free");
		}
	} else {
		const int64_t ntot = nt + nfree;
		check(qpc_lgwz_run(prop, f.data(), nt + 1, &nt, &ntot), "qpc_lgwz_run");
	}
	check(qpc_lgwz_get(prop, c.data()), "qpc_lgwz_get");
	double norm = 0.0;
	check(qpc_lgwz_norm(prop, &norm), "qpc_lgwz_norm");
	qpc_lgwz_destroy(prop);
	c.push_back(norm);
	FILE* o = std::fopen(argv[10], "wb");
	if (!o || std::fwrite(c.data(), sizeof(double), c.size(), o) != c.size()) { std::fprintf(stderr, "cannot write %s\n", argv[10]); return 2; }
	std::fclose(o);
	std::printf("norm %.16f\n", norm);
	return 0;
}
