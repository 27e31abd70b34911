// Harness that drives the UNMODIFIED reference headers (QPC-TDSE include/, read
// in place from the reference checkout) to produce golden vectors for the
// oracle and to time the reference's own CPU propagator.
//
// Test infrastructure, not product code.  Built by oracle/ref/Makefile into
// oracle/_ref/ (never committed); only tests/golden/make_golden.py and the
// developer run it.  MKL, GSL and HDF5 are replaced by the headers in
// oracle/ref/shim/ (see their comments).
//
// Grid sizes are compile-time in the reference (dimension_1e<...>), so the
// Makefile builds one binary per grid with -DHNR (active B-splines),
// -DHMR (B-spline degree p), -DHNL (number of l channels per m), -DHNM (number
// of m channels) and -DHM0 (first m).
//
// Commands (all arrays are written as raw little-endian float64 files):
//   setup  OUT RMAX DT ZC ZS SG
//       S, R (=<B|r|B>), RINV, D (=<B|d/dr|B>), H[l] for l=0..NL-1, the CN bands
//       upper/lower (lower already LDL^T-factorised by lu_zsb), the Cholesky factor
//       of S (operator_sc::initialize, operators/1e.hpp:1233-1244), the Y10 eigen-
//       system yeig[L], yprj[L][L], the knot vector, ground state (l=0, n=0).
//       Follows binsrc/sphTDSE.cpp:742-743 and cn_1e.hpp:565-593.
//   field  OUT E0 W0 NC N0 CEP DT
//       f(t_i) for i = 0..para_nt of field<field_component_sinen<2>> on 'z',
//       as binsrc/sphTDSE.cpp:738 and structure/field.h:229-311.
//   propagate OUT RMAX DT ZC ZS SG INIT FIELD NT NFREE NTHREADS
//       INIT = "gs" (ground state, l=0) or a file of 2*L*NR doubles; FIELD = file
//       of NT+1 doubles f(t_0..t_NT).  Runs propagate(coef, f[i], f[i+1]) for
//       i < NT, then NFREE field-free steps (binsrc/sphTDSE.cpp:786-831 loop
//       without observe/mask), and writes coef, S-norm, <z> (observable_z with
//       f(r)=r) and the wall time of the step loop (qpc::timer semantics).
//   arnoldi OUT RMAX DT ZC ZS SG INIT FIELD NT KMAX EMIN EMAX
//       NT steps of the Arnoldi propagator propagator_hc_lgwz (la_1e.hpp:390-444)
//       with ez = FIELD[i] during step i; see cmd_arnoldi.
//   vgwr   OUT RMAX DT ZC ZS SG INIT FIELD NT NFREE
//       the velocity-gauge elliptical propagator propagator_cn_hc_vgwr
//       (cn_1e.hpp:812-951): FIELD holds NT+1 rows (A_x, A_y) at t_0..t_NT; runs
//       propagate(coef, ax_i, ax_i+1, ay_i, ay_i+1) for i < NT, then NFREE field-free
//       steps; writes coef, the S-norm, the eigenvalues of the four couplings and the
//       dipole <x>, <y> before every step (observable_r, the elliptical driver's record).
//   mask   OUT RMAX DT ZC ZS SG INIT RMIN RMAXM INDEX
//       absorber_mask (absorber.hpp:40-63) initialised on [RMIN, RMAXM] with exponent INDEX
//       and applied once to INIT: writes the mask band and the masked coefficients.
//   proj   OUT RMAX DT ZC ZS SG COEF EMAX
//       Projection of COEF onto field-free eigenstates with E < EMAX
//       (eigenstate_sph::initialize + projection, population_1e.hpp:29-118).
//   pcs    OUT RMAX DT ZC ZS SG COEF KRMIN KRMAX THMIN THMAX PHMIN PHMAX PZC RB FLAG
//   tsurff OUT RMAX DT ZC ZS SG INIT FIELD NT NFREE MODE R0 TZC KRMIN KRMAX THMIN THMAX PHMIN PHMAX FLAG
//   pcsnum OUT RMAX DT ZC ZS SG COEF KRMIN KRMAX THMIN THMAX PHMIN PHMAX FLAG
//       momentum spectra (spectrum/momentum_1e.hpp); see cmd_pcs, cmd_tsurff and cmd_pcsnum.
#include <spherical/inventory.h>
#include <omp.h>
#include <string>
#include <vector>
#include <cstring>
#include <cstdlib>

using namespace qpc;
using namespace qpc::spherical;

#ifndef HNR
#define HNR 64
#endif
#ifndef HMR
#define HMR 6
#endif
#ifndef HNL
#define HNL 6
#endif
#ifndef HNM
#define HNM 1
#endif
#ifndef HM0
#define HM0 0
#endif

using dims_t = dimension_1e<HNR, HMR, HNL, HNM, HM0>;

static void dump(const std::string& dir, const char* name, const void* p, size_t ndouble)
{
	std::string f = dir + "/" + name + ".bin";
	FILE* fp = std::fopen(f.c_str(), "wb");
	if (!fp) { std::perror(f.c_str()); std::exit(2); }
	std::fwrite(p, sizeof(double), ndouble, fp);
	std::fclose(fp);
}
static std::vector<double> slurp(const char* f, size_t ndouble)
{
	std::vector<double> v(ndouble);
	FILE* fp = std::fopen(f, "rb");
	if (!fp) { std::perror(f); std::exit(2); }
	if (std::fread(v.data(), sizeof(double), ndouble, fp) != ndouble) { std::fprintf(stderr, "short read %s\n", f); std::exit(2); }
	std::fclose(fp);
	return v;
}

struct potn_any
{
	double zc, zs, sg;
	double operator()(double r) const noexcept
	{
		if (zs == 0.0) return hydrogenic{zc}(r);
		return hydrogenic_yukawa{zc, zs, sg}(r);
	}
};

template <class prop_t>
static void init_prop(prop_t& prop, integrator_radi<dims_t>& radi, integrator_angu<dims_t>& angu, double rmax, double dt,
	const potn_any& potn, size_t nthd)
{
	radi.initialize(0.0, rmax);
	prop.initialize(nthd, radi, angu, 1.0, potn, dt);
}

static int cmd_setup(int argc, char** argv)
{
	if (argc < 8) return 1;
	std::string out = argv[2];
	double rmax = atof(argv[3]), dt = atof(argv[4]);
	potn_any potn{atof(argv[5]), atof(argv[6]), atof(argv[7])};
	auto radi = integrator_radi<dims_t>();
	auto angu = integrator_angu<dims_t>();
	auto prop = propagator_cn_hc_lgwz<dims_t>();
	init_prop(prop, radi, angu, rmax, dt, potn, 1);

	dump(out, "S", prop.s.sub(), dims_t::n_rsub);
	dump(out, "chol", prop.s.cholesky(), dims_t::n_rsub);
	dump(out, "R", prop.r.data, dims_t::n_rsub);
	{
		operator_rinv1<dims_t> ri; ri.initialize(radi); dump(out, "RINV", ri.data, dims_t::n_rsub);
		operator_rdif1<dims_t> d; d.initialize(radi); dump(out, "D", d.data, dims_t::n_rsub);
	}
	std::vector<double> h((dims_t::n_lmax + 1) * dims_t::n_rsub);
	for (size_t l = 0; l <= dims_t::n_lmax; ++l) std::memcpy(h.data() + l * dims_t::n_rsub, prop.h[l], sizeof(double) * dims_t::n_rsub);
	dump(out, "H", h.data(), h.size());
	dump(out, "upper", prop.prop_hc.upper.data, 2 * (dims_t::n_lmax + 1) * dims_t::n_rsub);
	dump(out, "lower", prop.prop_hc.lower.data, 2 * (dims_t::n_lmax + 1) * dims_t::n_rsub);
	dump(out, "yeig", prop.prop_z1.yeig.data, dims_t::m_dims * dims_t::l_dims);
	dump(out, "yprj", prop.tran_z1.yprj.data, dims_t::m_dims * dims_t::l_dims * dims_t::l_dims);
	dump(out, "y10", prop.y.data, dims_t::m_dims * dims_t::l_dims);
	{
		using base_t = typename integrator_radi<dims_t>::base_t;
		size_t nk = dims_t::nr + dims_t::mr + 3;
		dump(out, "knots", radi.base.knot() - 1, nk);
		(void)sizeof(base_t);
	}
	auto coef = coefficient<dims_t>();
	auto eng = coef.template initialize<1>(prop.s, prop.h, {0ul}, {0ul}, {0ul}, {comp_t{1.0}});
	dump(out, "gs_energy", eng.data(), 1);
	dump(out, "gs_coef", coef.data, 2 * dims_t::n_leng);
	return 0;
}

static int cmd_field(int argc, char** argv)
{
	if (argc < 9) return 1;
	std::string out = argv[2];
	std::array<std::array<double, 5>, 0> none{};
	std::array<std::array<double, 5>, 1> z{{{atof(argv[3]), atof(argv[4]), atof(argv[5]), atof(argv[6]), atof(argv[7])}}};
	double dt = atof(argv[8]);
	auto laser = create_laser_field<field_component_sinen<2>>(none, none, z, dt);
	std::vector<double> t(laser.para_nt + 1), f(laser.para_nt + 1);
	for (size_t i = 0; i <= laser.para_nt; ++i) { t[i] = laser.t(i); f[i] = std::get<2>(laser(t[i])); }
	double nt = (double)laser.para_nt;
	dump(out, "nt", &nt, 1);
	dump(out, "t", t.data(), t.size());
	dump(out, "f", f.data(), f.size());
	return 0;
}

static int cmd_propagate(int argc, char** argv)
{
	if (argc < 13) return 1;
	std::string out = argv[2];
	double rmax = atof(argv[3]), dt = atof(argv[4]);
	potn_any potn{atof(argv[5]), atof(argv[6]), atof(argv[7])};
	const char* init = argv[8];
	const char* field = argv[9];
	size_t nt = strtoul(argv[10], 0, 10), nfree = strtoul(argv[11], 0, 10);
	int nthd = atoi(argv[12]);
	omp_set_num_threads(nthd);
	auto radi = integrator_radi<dims_t>();
	auto angu = integrator_angu<dims_t>();
	auto prop = propagator_cn_hc_lgwz<dims_t>();
	init_prop(prop, radi, angu, rmax, dt, potn, nthd);
	auto coef = coefficient<dims_t>();
	if (std::string(init) == "gs") {
		coef.template initialize<1>(prop.s, prop.h, {0ul}, {0ul}, {0ul}, {comp_t{1.0}});
	} else {
		auto v = slurp(init, 2 * dims_t::n_leng);
		std::memcpy((double*)coef.data, v.data(), sizeof(double) * v.size());
	}
	std::vector<double> f = nt ? slurp(field, nt + 1) : std::vector<double>{};
	// optional per-step observation, as the driver does before each step (sphTDSE.cpp:794)
	const bool record = std::getenv("QPC_REF_RECORD_Z") != nullptr;
	auto obs_rec = observable_z<dims_t>();
	if (record) obs_rec.initialize(radi, angu);
	std::vector<double> zl;
	auto clock = timer();
	clock.tic();
	for (size_t it = 0; it < nt + nfree; ++it) {
		if (record) zl.push_back(obs_rec.observe(coef.data, coef.data)[0]);
		if (it < nt) prop.propagate(coef, f[it], f[it + 1]);
		else prop.propagate(coef);
	}
	clock.toc();
	double secs = clock.get();
	if (record) dump(out, "zlist", zl.data(), zl.size());
	double norm = 0.0;
	#pragma omp parallel
	{
		double part = 0.0;
		prop.s.observe(coef.data, part);
		#pragma omp atomic
		norm += part;
	}
	auto obs = observable_z<dims_t>();
	obs.initialize(radi, angu);
	comp_t zz = obs.observe(coef.data, coef.data);
	double z2[2] = {zz[0], zz[1]};
	dump(out, "coef", coef.data, 2 * dims_t::n_leng);
	dump(out, "norm", &norm, 1);
	dump(out, "dipole", z2, 2);
	dump(out, "seconds", &secs, 1);
	std::printf("steps %zu threads %d seconds %.6f\n", nt + nfree, nthd, secs);
	return 0;
}

static int cmd_proj(int argc, char** argv)
{
	if (argc < 10) return 1;
	std::string out = argv[2];
	double rmax = atof(argv[3]), dt = atof(argv[4]);
	potn_any potn{atof(argv[5]), atof(argv[6]), atof(argv[7])};
	auto v = slurp(argv[8], 2 * dims_t::n_leng);
	double emax = atof(argv[9]);
	auto radi = integrator_radi<dims_t>();
	auto angu = integrator_angu<dims_t>();
	auto prop = propagator_cn_hc_lgwz<dims_t>();
	init_prop(prop, radi, angu, rmax, dt, potn, 1);
	auto coef = coefficient<dims_t>();
	std::memcpy((double*)coef.data, v.data(), sizeof(double) * v.size());
	eigenstate_sph<dims_t> eig;
	eig.initialize(prop.s, prop.h, [emax](size_t, double e, const double*) { return e < emax; });
	std::vector<comp_t> proj; std::vector<size_t> size;
	eig.projection(coef, proj, size);
	std::vector<double> sz(size.begin(), size.end()), en;
	for (size_t l = 0; l < dims_t::l_dims; ++l) for (double e : eig.val(l)) en.push_back(e);
	dump(out, "proj", proj.data(), 2 * proj.size());
	dump(out, "proj_nnz", sz.data(), sz.size());
	dump(out, "proj_energy", en.data(), en.size());
	return 0;
}

// ---------------------------------------------------------------- Arnoldi (la_1e.hpp)
// The reference's propagator_hc_lgwz (la_1e.hpp:390-444) runs through the unmodified
// propagator_arnoldi::propagate1 (la_1e.hpp:312-335) but with a correct S^-1:
// operator_sc::inverse_all (operators/1e.hpp:1253-1260) steps i by n_dims and then
// offsets by i*n_dims, so it solves channels n_dims^2 apart.  fixed_sc solves each
// (m,l) channel with the reference's own inverse_sub (operators/1e.hpp:1247-1251).
namespace qpc { namespace spherical {
template <class dims_t>
struct fixed_sc {
	const operator_sc<dims_t>* s = nullptr;
	void observe(const comp_t* w, double& norm) const noexcept { s->observe(w, norm); }
	void inverse_all(comp_t* u) const noexcept
	{
		#pragma omp for
		for (size_t c = 0; c < dims_t::m_dims * dims_t::l_dims; ++c) s->inverse_sub(u + c * dims_t::n_dims);
	}
};
template <class dims_t>
struct type_of_inverse_all_t<fixed_sc<dims_t>> : public std::integral_constant<int, 0> {};

template <class dims_t>
struct harness_hc_lgwz : public propagator_hc_lgwz<dims_t> {
	fixed_sc<dims_t> oper_s;	// shadows the base's operator_sc for propagate1's CRTP lookup
	using propagator_hc_lgwz<dims_t>::propagator_hc_lgwz;
	int step(coefficient<dims_t>& w, double dt, size_t nthreads)
	{
		oper_s.s = &this->propagator_hc_lgwz<dims_t>::oper_s;
		return this->template propagate1<harness_hc_lgwz<dims_t>>(w, dt, nthreads);
	}
};
}}

//   arnoldi OUT RMAX DT ZC ZS SG INIT FIELD NT KMAX EMIN EMAX
//       NT Arnoldi steps of length DT with ez = FIELD[i] (NT values), from INIT
//       ("gs" or a file); writes coef and the criterion code of every step.
static int cmd_arnoldi(int argc, char** argv)
{
	if (argc < 14) return 1;
	std::string out = argv[2];
	double rmax = atof(argv[3]), dt = atof(argv[4]);
	potn_any potn{atof(argv[5]), atof(argv[6]), atof(argv[7])};
	const char* init = argv[8];
	const char* field = argv[9];
	size_t nt = strtoul(argv[10], 0, 10), kmax = strtoul(argv[11], 0, 10);
	double emin = atof(argv[12]), emax = atof(argv[13]);
	omp_set_num_threads(1);
	auto radi = integrator_radi<dims_t>();
	auto angu = integrator_angu<dims_t>();
	radi.initialize(0.0, rmax);
	auto prop = harness_hc_lgwz<dims_t>(kmax, emin, emax);
	prop.initialize(radi, angu, 1.0, potn);
	auto coef = coefficient<dims_t>();
	if (std::string(init) == "gs") {
		coef.template initialize<1>(prop.propagator_hc_lgwz<dims_t>::oper_s, prop.oper_h, {0ul}, {0ul}, {0ul}, {comp_t{1.0}});
	} else {
		auto v = slurp(init, 2 * dims_t::n_leng);
		std::memcpy((double*)coef.data, v.data(), sizeof(double) * v.size());
	}
	std::vector<double> f = slurp(field, nt), crit(nt);
	for (size_t it = 0; it < nt; ++it) {
		prop.ez = f[it];
		crit[it] = prop.step(coef, dt, 1);
	}
	dump(out, "coef", coef.data, 2 * dims_t::n_leng);
	dump(out, "crit", crit.data(), crit.size());
	return 0;
}

static int cmd_vgwr(int argc, char** argv)
{
	if (argc < 12) return 1;
	std::string out = argv[2];
	double rmax = atof(argv[3]), dt = atof(argv[4]);
	potn_any potn{atof(argv[5]), atof(argv[6]), atof(argv[7])};
	const char* init = argv[8];
	const char* field = argv[9];
	size_t nt = strtoul(argv[10], 0, 10), nfree = strtoul(argv[11], 0, 10);
	omp_set_num_threads(1);
	auto radi = integrator_radi<dims_t>();
	auto angu = integrator_angu<dims_t>();
	auto prop = propagator_cn_hc_vgwr<dims_t>();
	init_prop(prop, radi, angu, rmax, dt, potn, 1);
	auto coef = coefficient<dims_t>();
	auto v = slurp(init, 2 * dims_t::n_leng);
	std::memcpy((double*)coef.data, v.data(), sizeof(double) * v.size());
	std::vector<double> f = nt ? slurp(field, 2 * (nt + 1)) : std::vector<double>{};
	// the elliptical driver's observation before each step (binsrc/sphTDSE.cpp:515-527, 933):
	// observable_r with f(r) = r, x = Re(rm + rp)/2, y = Im(rp - rm)/2
	auto obs = observable_r<dims_t>();
	obs.initialize(radi, angu);
	std::vector<double> xs, ys;
	for (size_t it = 0; it < nt + nfree; ++it) {
		auto rm = obs.observe_rm(coef.data, coef.data);
		auto rp = obs.observe_rp(coef.data, coef.data);
		xs.push_back(real(rm + rp) / 2.0);
		ys.push_back(imag(rp - rm) / 2.0);
		if (it < nt) prop.propagate(coef, f[2 * it], f[2 * it + 2], f[2 * it + 1], f[2 * it + 3]);
		else prop.propagate(coef);
	}
	dump(out, "xlist", xs.data(), xs.size());
	dump(out, "ylist", ys.data(), ys.size());
	dump(out, "coef", coef.data, 2 * dims_t::n_leng);
	double norm = 0.0;
	#pragma omp parallel
	{
		double part = 0.0;
		prop.s.observe(coef.data, part);
		#pragma omp atomic
		norm += part;
	}
	dump(out, "norm", &norm, 1);
	const size_t nc = dims_t::m_dims * dims_t::l_dims;
	dump(out, "zeig_x1", prop.prop_x1.zeig.data, nc);
	dump(out, "zeig_x2", prop.prop_x2.zeig.data, nc);
	dump(out, "zeig_y1", prop.prop_y1.zeig.data, nc);
	dump(out, "zeig_y2", prop.prop_y2.zeig.data, nc);
	return 0;
}

static int cmd_mask(int argc, char** argv)
{
	if (argc < 12) return 1;
	std::string out = argv[2];
	double rmax = atof(argv[3]), dt = atof(argv[4]);
	potn_any potn{atof(argv[5]), atof(argv[6]), atof(argv[7])};
	const char* init = argv[8];
	double r0 = atof(argv[9]), r1 = atof(argv[10]), index = atof(argv[11]);
	omp_set_num_threads(1);
	auto radi = integrator_radi<dims_t>();
	auto angu = integrator_angu<dims_t>();
	auto prop = propagator_cn_hc_lgwz<dims_t>();
	init_prop(prop, radi, angu, rmax, dt, potn, 1);
	auto coef = coefficient<dims_t>();
	auto v = slurp(init, 2 * dims_t::n_leng);
	std::memcpy((double*)coef.data, v.data(), sizeof(double) * v.size());
	struct probe : absorber_mask<dims_t> {
		using absorber_mask<dims_t>::absorber_mask;
		const double* band() const { return this->data; }
	};
	auto mask = probe(1);
	mask.initialize(radi, r0, r1, index);
	coefficient_view<dims_t> view{coef.data};
	mask(view, prop.s);
	dump(out, "maskband", mask.band(), dims_t::n_rsub);
	dump(out, "coef", coef.data, 2 * dims_t::n_leng);
	return 0;
}

// ---------------------------------------------------------------- momentum spectra (momentum_1e.hpp)
// Momentum grids are compile-time in the reference (spectrum_c_pcs<dims_t, nkr, nkt, nkp>):
// -DHNKR, -DHNKT, -DHNKP.
#ifndef HNKR
#define HNKR 24
#endif
#ifndef HNKT
#define HNKT 5
#endif
#ifndef HNKP
#define HNKP 4
#endif

//   pcs OUT RMAX DT ZC ZS SG COEF KRMIN KRMAX THMIN THMAX PHMIN PHMAX PZC RB FLAG
//       spectrum_c_pcs::initialize with the analytic Coulomb waves of charge PZC and cut-off RB
//       (momentum_1e.hpp:453-485) on the grid of RMAX, then measure_lmd, measure_prj and
//       measure_pad of COEF (337-403); writes the axes, the tables and the three spectra.
static int cmd_pcs(int argc, char** argv)
{
	if (argc < 18) return 1;
	std::string out = argv[2];
	double rmax = atof(argv[3]);
	const char* cf = argv[8];
	double krmin = atof(argv[9]), krmax = atof(argv[10]), thmin = atof(argv[11]), thmax = atof(argv[12]);
	double phmin = atof(argv[13]), phmax = atof(argv[14]), pzc = atof(argv[15]), rb = atof(argv[16]);
	int flag = atoi(argv[17]);
	omp_set_num_threads(1);
	auto radi = integrator_radi<dims_t>();
	radi.initialize(0.0, rmax);
	auto coef = coefficient<dims_t>();
	auto v = slurp(cf, 2 * dims_t::n_leng);
	std::memcpy((double*)coef.data, v.data(), sizeof(double) * v.size());
	coefficient_view<dims_t> view{coef.data};
	auto* pcs = new spectrum_c_pcs<dims_t, HNKR, HNKT, HNKP>();
	pcs->initialize(radi, krmin, krmax, thmin, thmax, phmin, phmax, pzc, rb, flag);
	dump(out, "kr", pcs->kr, HNKR);
	dump(out, "kt", pcs->kt, HNKT);
	dump(out, "kp", pcs->kp, HNKP);
	dump(out, "ijl", pcs->ijl.data, pcs->ijl.dim.n_leng);
	dump(out, "plm", pcs->plm.data, pcs->plm.dim.n_leng);
	dump(out, "exm", pcs->exm.data, 2 * pcs->exm.dim.n_leng);
	dump(out, "cps", pcs->cps.data, 2 * pcs->cps.dim.n_leng);
	pcs->measure_lmd(view, 1);
	dump(out, "lmd", pcs->dptr(), 2 * pcs->size());
	pcs->measure_prj(view, 1);
	dump(out, "pmd", pcs->dptr(), 2 * pcs->size());
	pcs->measure_pad(view, 1);
	dump(out, "pad", pcs->dptr(), 2 * pcs->size());
	delete pcs;
	return 0;
}

//   pcsnum OUT RMAX DT ZC ZS SG COEF KRMIN KRMAX THMIN THMAX PHMIN PHMAX FLAG
//       spectrum_c_pcs::initialize with the numerical partial waves of V = -(ZC + ZS e^{-SG r})/r
//       (generate_odefun_from_potential, the driver's choice for screened potentials,
//       binsrc/sphTDSE.cpp:313-316, 340-342), then the three measurements of COEF.
static int cmd_pcsnum(int argc, char** argv)
{
	if (argc < 16) return 1;
	std::string out = argv[2];
	double rmax = atof(argv[3]);
	double zc = atof(argv[5]), zs = atof(argv[6]), sg = atof(argv[7]);
	const char* cf = argv[8];
	double krmin = atof(argv[9]), krmax = atof(argv[10]), thmin = atof(argv[11]), thmax = atof(argv[12]);
	double phmin = atof(argv[13]), phmax = atof(argv[14]);
	int flag = atoi(argv[15]);
	omp_set_num_threads(1);
	auto radi = integrator_radi<dims_t>();
	radi.initialize(0.0, rmax);
	auto coef = coefficient<dims_t>();
	auto v = slurp(cf, 2 * dims_t::n_leng);
	std::memcpy((double*)coef.data, v.data(), sizeof(double) * v.size());
	coefficient_view<dims_t> view{coef.data};
	auto* pcs = new spectrum_c_pcs<dims_t, HNKR, HNKT, HNKP>();
	if (zs != 0.0) {
		auto odef = generate_odefun_from_potential(hydrogenic_yukawa{zc, zs, sg}, 1.0);
		pcs->initialize(radi, krmin, krmax, thmin, thmax, phmin, phmax, odef, flag);
	} else {
		auto odef = generate_odefun_from_potential(hydrogenic{zc}, 1.0);
		pcs->initialize(radi, krmin, krmax, thmin, thmax, phmin, phmax, odef, flag);
	}
	dump(out, "kr", pcs->kr, HNKR);
	dump(out, "ijl", pcs->ijl.data, pcs->ijl.dim.n_leng);
	dump(out, "cps", pcs->cps.data, 2 * pcs->cps.dim.n_leng);
	pcs->measure_lmd(view, 1);
	dump(out, "lmd", pcs->dptr(), 2 * pcs->size());
	pcs->measure_prj(view, 1);
	dump(out, "pmd", pcs->dptr(), 2 * pcs->size());
	delete pcs;
	return 0;
}

//   tsurff OUT RMAX DT ZC ZS SG INIT FIELD NT NFREE MODE R0 TZC KRMIN KRMAX THMIN THMAX PHMIN PHMAX FLAG
//       spectrum_c_tsf::initialize at R0 with Coulomb correction TZC (momentum_1e.hpp:778-866), then the
//       driver loop with t-SURFF (binsrc/sphTDSE.cpp:786-831, 936-945): MODE "z" propagates with
//       propagator_cn_hc_lgwz and FIELD = NT+1 values f_i, calling accumulate(f_i, f_i+1, dt, coef)
//       after each field step; MODE "xy" with propagator_cn_hc_vgwr and FIELD = NT+1 rows (A_x, A_y),
//       calling accumulate(ax_i, ax_i+1, ay_i, ay_i+1, dt, coef); both call accumulate(dt, coef) after
//       each of the NFREE field-free steps.  Writes the tables, the spectrum work and the final coef.
static int cmd_tsurff(int argc, char** argv)
{
	if (argc < 21) return 1;
	std::string out = argv[2];
	double rmax = atof(argv[3]), dt = atof(argv[4]);
	potn_any potn{atof(argv[5]), atof(argv[6]), atof(argv[7])};
	const char* init = argv[8];
	const char* field = argv[9];
	size_t nt = strtoul(argv[10], 0, 10), nfree = strtoul(argv[11], 0, 10);
	std::string mode = argv[12];
	double r0 = atof(argv[13]), tzc = atof(argv[14]);
	double krmin = atof(argv[15]), krmax = atof(argv[16]), thmin = atof(argv[17]), thmax = atof(argv[18]);
	double phmin = atof(argv[19]), phmax = atof(argv[20]);
	int flag = argc > 21 ? atoi(argv[21]) : 0;
	if (mode != "z" && mode != "xy") return 1;
	omp_set_num_threads(1);
	auto radi = integrator_radi<dims_t>();
	auto angu = integrator_angu<dims_t>();
	auto coef = coefficient<dims_t>();
	auto v = slurp(init, 2 * dims_t::n_leng);
	std::memcpy((double*)coef.data, v.data(), sizeof(double) * v.size());
	auto* tsf = new spectrum_c_tsf<dims_t, HNKR, HNKT, HNKP>();
	radi.initialize(0.0, rmax);
	tsf->initialize(radi, angu, r0, tzc, krmin, krmax, thmin, thmax, phmin, phmax, flag);
	if (mode == "z") {
		auto prop = propagator_cn_hc_lgwz<dims_t>();
		prop.initialize(1, radi, angu, 1.0, potn, dt);
		std::vector<double> f = nt ? slurp(field, nt + 1) : std::vector<double>{};
		for (size_t it = 0; it < nt + nfree; ++it) {
			if (it < nt) { prop.propagate(coef, f[it], f[it + 1]); tsf->accumulate(f[it], f[it + 1], dt, coef.data); }
			else { prop.propagate(coef); tsf->accumulate(dt, coef.data); }
		}
	} else {
		auto prop = propagator_cn_hc_vgwr<dims_t>();
		prop.initialize(1, radi, angu, 1.0, potn, dt);
		std::vector<double> f = nt ? slurp(field, 2 * (nt + 1)) : std::vector<double>{};
		for (size_t it = 0; it < nt + nfree; ++it) {
			if (it < nt) {
				prop.propagate(coef, f[2 * it], f[2 * it + 2], f[2 * it + 1], f[2 * it + 3]);
				tsf->accumulate(f[2 * it], f[2 * it + 2], f[2 * it + 1], f[2 * it + 3], dt, coef.data);
			} else { prop.propagate(coef); tsf->accumulate(dt, coef.data); }
		}
	}
	dump(out, "kr", tsf->kr, HNKR);
	dump(out, "kt", tsf->kt, HNKT);
	dump(out, "kp", tsf->kp, HNKP);
	std::vector<double> ibd(tsf->ib, tsf->ib + tsf->nb);
	dump(out, "ib", ibd.data(), ibd.size());
	dump(out, "b0", tsf->b0, tsf->nb);
	dump(out, "br", tsf->br, tsf->nb);
	dump(out, "j0", tsf->j0.data, tsf->j0.dim.n_leng);
	dump(out, "jr", tsf->jr.data, tsf->jr.dim.n_leng);
	dump(out, "y0", tsf->y0.data, tsf->y0.dim.n_leng);
	dump(out, "e0", tsf->e0.data, 2 * tsf->e0.dim.n_leng);
	dump(out, "pmat0", tsf->pmat0.data, tsf->pmat0.dim.n_leng);
	dump(out, "pmat1", tsf->pmat1.data, tsf->pmat1.dim.n_leng);
	dump(out, "pmat2", tsf->pmat2.data, tsf->pmat2.dim.n_leng);
	dump(out, "work", tsf->dptr(), 2 * tsf->size());
	double clk[4] = {tsf->time, tsf->disx, tsf->disy, tsf->disz};
	dump(out, "clock", clk, 4);
	dump(out, "coef", coef.data, 2 * dims_t::n_leng);
	delete tsf;
	return 0;
}

int main(int argc, char** argv)
{
	if (argc < 2) { std::fprintf(stderr, "usage: setup|field|propagate|proj|arnoldi ...\n"); return 1; }
	try {
		std::string c = argv[1];
		int rc = 1;
		if (c == "setup") rc = cmd_setup(argc, argv);
		else if (c == "field") rc = cmd_field(argc, argv);
		else if (c == "propagate") rc = cmd_propagate(argc, argv);
		else if (c == "proj") rc = cmd_proj(argc, argv);
		else if (c == "arnoldi") rc = cmd_arnoldi(argc, argv);
		else if (c == "vgwr") rc = cmd_vgwr(argc, argv);
		else if (c == "mask") rc = cmd_mask(argc, argv);
		else if (c == "pcs") rc = cmd_pcs(argc, argv);
		else if (c == "tsurff") rc = cmd_tsurff(argc, argv);
		else if (c == "pcsnum") rc = cmd_pcsnum(argc, argv);
		if (rc) std::fprintf(stderr, "bad arguments for %s\n", argv[1]);
		return rc;
	} catch (std::exception& e) {
		std::fprintf(stderr, "reference threw: %s\n", e.what());
		return 3;
	}
}
