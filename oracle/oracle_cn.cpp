// CPU oracle for the QPC-TDSE length-gauge Crank-Nicolson time step.
//
// TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg load this library, as the checker and as the
// timed CPU stand-in for the reference.  The GPU product never links it.
//
// It restates, in plain C++ with OpenMP, the arithmetic of the reference's
// propagator_cn_hc_lgwz, in the reference's own order of operations:
//   * complex multiply / divide as qpc::avx128_complex does them
//     (libraries/avx/avx128_complex.h:38-95): x*y = (fma(yr,xr,-yi*xi),
//     fma(yr,xi,yi*xr)); x/y = (fma(yr,xr,yi*xi), fma(yr,xi,-yi*xr)) /
//     fma(yr,yr,yi*yi); 1/y = (yr,-yi) / (yr*yr + yi*yi).
//   * lu_zsb, the in-place complex-symmetric banded LDL^T (algorithm/ed.h:208-289).
//   * cn_component_hc::initialize, upper = S - i dt/2 H_l, lower = LDL^T of
//     S + i dt/2 H_l (spherical/propagator/cn_1e.hpp:342-360).
//   * cn_hc_propagate0, w = upper c, w = L^-1 w, c = (D L^T)^-1 w
//     (spherical/propagator/propagate.hpp:311-331, utilities/blas2.hpp:452-508,
//     1058-1108 and the loop kernels at 435-447).
//   * cn_propagate_kernel_avx1<0>, the on-the-fly banded LU of S + a R fused
//     with y = L^-1 (S - a R) z, then z = U^-1 y (propagate.hpp:3-98), with
//     a = i lambda f dt/4 (propagate.hpp:343, cn_1e.hpp:409-415, 588).
//   * cn_transform_hl<double>::construct/eliminate, tmp[m] = P[m] c[m] and
//     c[m] = P[m]^T tmp[m] with P real, rows = eigenvectors of Y10
//     (cn_1e.hpp:101-147).
//   * propagator_cn_hc_lgwz::propagate, coupling(f_ti) -> field-free ->
//     coupling(f_tf), and the field-free-only overload (cn_1e.hpp:595-618).
//   * the S-norm (operators/1e.hpp:69-89 with symb_prj_vecd, blas2.hpp:1109-1127)
//     and <cos(theta) f(r)> (observable/1e.hpp:26-50).
// Compiled with -ffp-contract=off so that only the fma() calls written here fuse.
//
// Layout everywhere: state [inst][m][l][r] complex128 (re, im interleaved);
// symmetric bands in upper-row form band[r*(p+1)+k] = A(r, r+k).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <omp.h>

namespace {

struct cx { double re, im; };

inline cx cadd(cx a, cx b) { return {a.re + b.re, a.im + b.im}; }
inline cx csub(cx a, cx b) { return {a.re - b.re, a.im - b.im}; }
// avx_mul(x, y): fmaddsub(yr, x, yi * swap(x))
inline cx cmul(cx x, cx y) { return {std::fma(y.re, x.re, -(y.im * x.im)), std::fma(y.re, x.im, y.im * x.re)}; }
inline cx cmul(cx x, double y) { return {x.re * y, x.im * y}; }
// avx_div(x, y)
inline cx cdiv(cx x, cx y)
{
	double nr = std::fma(y.re, x.re, y.im * x.im);
	double ni = std::fma(y.re, x.im, -(y.im * x.re));
	double d = std::fma(y.re, y.re, y.im * y.im);
	return {nr / d, ni / d};
}
// avx_div(double x, complex y)
inline cx crcp(double x, cx y)
{
	double d0 = y.re * y.re + y.im * y.im;
	double d1 = y.im * y.im + y.re * y.re;
	return {(x * y.re) / d0, (-x * y.im) / d1};
}
inline double cnorm(cx x) { return x.re * x.re + x.im * x.im; }

inline long lof(int im, int il, int m0) { long m = (long)im + m0; return (long)il + (m < 0 ? -m : m); }

// ---------------------------------------------------------------- lu_zsb (ed.h:208-289)
int lu_zsb(int n, int p, cx* a)
{
	const int ne = p + 1;
	int info = 0;
	auto kernel = [&](cx* ar, int kmax) {
		for (int k = 1; k < kmax; ++k) {
			cx* as = ar - (long)p * k;
			cx aa = cmul(as[0], as[-k]);
			for (int i = 0; i < ne - k; ++i) ar[i] = csub(ar[i], cmul(aa, as[i]));
		}
		if (cnorm(ar[0]) < 1e-31) info++;
		cx a0 = crcp(1.0, ar[0]);
		for (int i = 1; i < ne; ++i) ar[i] = cmul(ar[i], a0);
	};
	for (int j = 0; j < ne; ++j) kernel(a + (long)j * ne, 1 + j);
	for (int j = ne; j < n - p; ++j) kernel(a + (long)j * ne, ne);
	for (int j = n - p; j < n; ++j) {
		for (int i = n - j; i < ne; ++i) a[(long)j * ne + i] = {0.0, 0.0};
		kernel(a + (long)j * ne, ne);
	}
	return info;
}

// ---------------------------------------------------------------- field-free CN (propagate.hpp:311-331)
void hc_channel(int n, int p, const cx* up, const cx* lo, cx* c, cx* w)
{
	const int m = p + 1, q = p;
	// w = up * c  (symb_mul_vecd<n,m,0>, 2m <= n branch)
	for (int i = 0; i < n; ++i) {
		int jmax = std::min(i + 1, m), kmax = std::min(m, n - i);
		const cx* a = up + (long)i * m;
		const cx* x = c + i;
		cx t = {0.0, 0.0};
		for (int j = 1; j < jmax; ++j) t = cadd(t, cmul(a[-(long)j * q], x[-j]));
		for (int k = 0; k < kmax; ++k) t = cadd(t, cmul(a[k], x[k]));
		w[i] = t;
	}
	// w = L^-1 w (ltrb_ldl_vecd): j descending
	for (int i = 0; i < n; ++i) {
		int jmax = std::min(i + 1, m);
		const cx* a = lo + (long)i * m;
		cx x = w[i];
		for (int j = jmax; j-- > 1;) x = csub(x, cmul(w[i - j], a[-(long)j * q]));
		w[i] = x;
	}
	// c = (D L^T)^-1 w (utrb_ldl_vecd)
	for (int i = 0; i < n; ++i) {
		int s = n - 1 - i;
		int kmax = std::min(i + 1, m);
		const cx* a = lo + (long)s * m;
		cx x = cdiv(w[s], a[0]);
		for (int k = 1; k < kmax; ++k) x = csub(x, cmul(c[s + k], a[k]));
		c[s] = x;
	}
}

// ---------------------------------------------------------------- coupling CN (propagate.hpp:3-98), symflag 0 or 1
void cn_channel(int n, int p, const double* smat, const double* rmat, cx ifet, cx* z, cx* y, cx* u, bool anti = false)
{
	const int ne = p + 1;
	cx a[2 * 16 + 1], b[2 * 16 + 1];
	for (int i = 0; i < n; ++i) {
		for (int j = 1; j < ne; ++j) {
			long k = (long)i * ne - (long)j * p;
			int _j = p - j;
			if (i < j) { a[_j] = {0, 0}; b[_j] = {0, 0}; }
			else {
				double s = smat[k], r = rmat[k];
				cx fr = cmul(ifet, r);
				// symflag = 1: r is the upper entry of an anti-symmetric band (propagate.hpp:45-47)
				a[_j] = anti ? cadd({s, 0.0}, fr) : csub({s, 0.0}, fr);
				b[_j] = anti ? csub({s, 0.0}, fr) : cadd({s, 0.0}, fr);
			}
		}
		for (int j = 0; j < ne; ++j) {
			long k = (long)i * ne + j;
			double s = smat[k], r = rmat[k];
			cx fr = cmul(ifet, r);
			a[p + j] = csub({s, 0.0}, fr);
			b[p + j] = cadd({s, 0.0}, fr);
		}
		int l = p > i ? p - i : 0;
		int h = (n - 1 - p > i) ? 2 * p + 1 : p + n - i;
		for (int j = l; j < p; ++j)
			for (int k = 0; k < p; ++k) b[j + k + 1] = csub(b[j + k + 1], cmul(b[j], u[(long)(i + j - p) * p + k]));
		for (int j = 0; j < p; ++j) u[(long)i * p + j] = cdiv(b[j + p + 1], b[p]);
		cx v = {0, 0};
		for (int j = l; j < h; ++j) v = cadd(v, cmul(a[j], z[i + j - p]));
		for (int j = l; j < p; ++j) v = csub(v, cmul(b[j], y[i + j - p]));
		y[i] = cdiv(v, b[p]);
	}
	for (int i = n; i-- > 0;) {
		int jmax = std::min(ne, n - i);
		cx v = {0, 0};
		for (int j = 1; j < jmax; ++j) v = cadd(v, cmul(y[i + j], u[(long)i * p + j - 1]));
		y[i] = csub(y[i], v);
		z[i] = y[i];
	}
}

} // namespace

extern "C" {

struct oracle_lgwz {
	int32_t n_r, p, n_l, n_m, m0, n_inst;
	double dt;
	const double* S;     // [n_r][p+1]
	const double* R;     // [n_r][p+1]
	const double* yeig;  // [n_m][n_l]
	const double* yprj;  // [n_m][n_l][n_l], row a = eigenvector a
	const double* upper; // [lmax+1][n_r][p+1] complex
	const double* lower; // [lmax+1][n_r][p+1] complex, LDL^T factorised
};

int oracle_lu_zsb(int n, int p, double* band) { return lu_zsb(n, p, (cx*)band); }

// upper = S - i dt/2 H_l, lower = lu_zsb(S + i dt/2 H_l) for l = 0..nl-1 (cn_1e.hpp:342-360)
int oracle_cn_bands(int n, int p, int nl, const double* S, const double* H, double dt, double* upper, double* lower)
{
	const long nrs = (long)n * (p + 1);
	int err = 0;
	for (int l = 0; l < nl; ++l) {
		cx* up = (cx*)upper + l * nrs;
		cx* lo = (cx*)lower + l * nrs;
		for (long i = 0; i < nrs; ++i) {
			double si = S[i];
			// hi = h*unim*dt*0.5 : (h*(0,1)) -> (0*h, 1*h) then *dt then *0.5
			cx hi = {0.0 * H[l * nrs + i], 1.0 * H[l * nrs + i]};
			hi = cmul(cmul(hi, dt), 0.5);
			up[i] = csub({si, 0.0}, hi);
			lo[i] = cadd({si, 0.0}, hi);
		}
		err += lu_zsb(n, p, lo);
	}
	return err;
}

static void transform(const oracle_lgwz* g, const cx* src, cx* dst, bool transpose)
{
	const int L = g->n_l, N = g->n_r;
	const long ch = (long)g->n_m * g->n_inst;
	#pragma omp for schedule(static)
	for (long im = 0; im < ch; ++im) {
		const double* P = g->yprj + (im % g->n_m) * (long)L * L;
		const cx* s = src + im * L * (long)N;
		cx* d = dst + im * L * (long)N;
		// d[a][r] = sum_b w(a,b) s[b][r], b ascending for every (a, r)
		for (int a = 0; a < L; ++a) {
			cx* da = d + (long)a * N;
			for (int r = 0; r < N; ++r) da[r] = {0.0, 0.0};
			for (int b = 0; b < L; ++b) {
				double w = transpose ? P[(long)b * L + a] : P[(long)a * L + b];
				const cx* sb = s + (long)b * N;
				for (int r = 0; r < N; ++r) { da[r].re += w * sb[r].re; da[r].im += w * sb[r].im; }
			}
		}
	}
}

static void coupling(const oracle_lgwz* g, cx* tmp, const double* f)
{
	const int N = g->n_r, p = g->p;
	const long nch = (long)g->n_inst * g->n_m * g->n_l;
	thread_local std::vector<cx> y, u;
	if ((long)y.size() < N) y.resize(N);
	if ((long)u.size() < (long)N * p) u.resize((long)N * p);
	#pragma omp for schedule(static)
	for (long c = 0; c < nch; ++c) {
		long inst = c / ((long)g->n_m * g->n_l);
		long iml = c % ((long)g->n_m * g->n_l);
		double fzdt = f[inst] * (g->dt * 0.5);
		cx ifdt = {0.0 * (fzdt / 2), 1.0 * (fzdt / 2)};
		cx ifet = cmul(ifdt, g->yeig[iml]);
		cn_channel(N, p, g->S, g->R, ifet, tmp + c * N, y.data(), u.data());
	}
}

static void fieldfree(const oracle_lgwz* g, cx* coef)
{
	const int N = g->n_r, p = g->p;
	const long nrs = (long)N * (p + 1);
	const long nch = (long)g->n_inst * g->n_m * g->n_l;
	thread_local std::vector<cx> w;
	if ((long)w.size() < N) w.resize(N);
	#pragma omp for schedule(static)
	for (long c = 0; c < nch; ++c) {
		long iml = c % ((long)g->n_m * g->n_l);
		long l = lof((int)(iml / g->n_l), (int)(iml % g->n_l), g->m0);
		hc_channel(N, p, (const cx*)g->upper + l * nrs, (const cx*)g->lower + l * nrs, coef + c * N, w.data());
	}
}

// One propagator_cn_hc_lgwz::propagate(coef, f_ti, f_tf) per instance (f_ti == NULL: field-free step).
void oracle_lgwz_step(const oracle_lgwz* g, double* coef, const double* f_ti, const double* f_tf, int nthreads)
{
	const long len = (long)g->n_inst * g->n_m * g->n_l * g->n_r;
	thread_local std::vector<cx> tmp;
	if (f_ti && (long)tmp.size() < len) tmp.resize(len);
	cx* c = (cx*)coef;
	#pragma omp parallel num_threads(nthreads) if (nthreads > 1)
	{
		if (f_ti) {
			transform(g, c, tmp.data(), false);
			coupling(g, tmp.data(), f_ti);
			transform(g, tmp.data(), c, true);
		}
		fieldfree(g, c);
		if (f_ti) {
			transform(g, c, tmp.data(), false);
			coupling(g, tmp.data(), f_tf);
			transform(g, tmp.data(), c, true);
		}
	}
}

// The driver loop of binsrc/sphTDSE.cpp:786-831 for a batch whose instances share
// one grid: instance k takes nt_field[k] field steps with f(t_i) = ftab[k*ld + i]
// then field-free steps until nt_total[k].  Instances run independently
// (one OpenMP thread each), which is how the reference runs many wavefunctions:
// many independent processes.
void oracle_lgwz_run(const oracle_lgwz* g, double* coef, const double* ftab, long ld, const int64_t* nt_field,
	const int64_t* nt_total, int nthreads)
{
	const long per = (long)g->n_m * g->n_l * g->n_r;
	#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
	for (long k = 0; k < g->n_inst; ++k) {
		oracle_lgwz one = *g;
		one.n_inst = 1;
		for (int64_t it = 0; it < nt_total[k]; ++it) {
			if (it < nt_field[k]) oracle_lgwz_step(&one, coef + 2 * k * per, ftab + k * ld + it, ftab + k * ld + it + 1, 1);
			else oracle_lgwz_step(&one, coef + 2 * k * per, nullptr, nullptr, 1);
		}
	}
}

// x^H A y for symmetric band A (symb_prj_vecd_naive, blas2.hpp:1109-1127)
static cx prj(int n, int p, const double* A, const cx* x, const cx* y)
{
	const int m = p + 1, q = p;
	cx tmp = {0, 0};
	for (int i = 0; i < n; ++i) {
		int jmax = std::min(i + 1, m), kmax = std::min(m, n - i);
		const double* a = A + (long)i * m;
		cx t = {0, 0};
		for (int j = 1; j < jmax; ++j) t = cadd(t, cmul(y[i - j], a[-(long)j * q]));
		for (int k = 0; k < kmax; ++k) t = cadd(t, cmul(y[i + k], a[k]));
		// avx_mulc(t, x) = t * conj(x)
		tmp = cadd(tmp, cx{std::fma(x[i].re, t.re, x[i].im * t.im), std::fma(x[i].re, t.im, -(x[i].im * t.re))});
	}
	return tmp;
}

// S-norm per instance: sum over (m,l) of Re c^H S c (operators/1e.hpp:69-89)
void oracle_norm(const oracle_lgwz* g, const double* coef, double* out)
{
	const long per = (long)g->n_m * g->n_l;
	for (long k = 0; k < g->n_inst; ++k) {
		double s = 0;
		for (long c = 0; c < per; ++c) {
			const cx* w = (const cx*)coef + (k * per + c) * g->n_r;
			s += prj(g->n_r, g->p, g->S, w, w).re;
		}
		out[k] = s;
	}
}

// <c| cos(theta) f(r) |c> per instance with band F = <B|f|B> and y10(m,l)
// (observable_z::observe, observable/1e.hpp:26-50); out[2k], out[2k+1] = re, im.
void oracle_dipole(const oracle_lgwz* g, const double* F, const double* y10, const double* coef, double* out)
{
	const int L = g->n_l, N = g->n_r;
	const long per = (long)g->n_m * L;
	for (long k = 0; k < g->n_inst; ++k) {
		cx s = {0, 0};
		for (int im = 0; im < g->n_m; ++im)
			for (int il = 0; il < L; ++il) {
				const cx* base = (const cx*)coef + (k * per + (long)im * L) * N;
				if (il > 0) s = cadd(s, cmul(prj(N, g->p, F, base + (long)il * N, base + (long)(il - 1) * N), y10[im * L + il - 1]));
				if (il + 1 < L) s = cadd(s, cmul(prj(N, g->p, F, base + (long)il * N, base + (long)(il + 1) * N), y10[im * L + il]));
			}
		out[2 * k] = s.re;
		out[2 * k + 1] = s.im;
	}
}

// ---------------------------------------------------------------- velocity gauge, elliptical
// propagator_cn_hc_vgwr::propagate (cn_1e.hpp:903-945): four coupling components, each a
// dense (m,l) transform and one banded CN per eigen-channel, around the field-free step.
//   x1: P_x1 (real), cn_hm_propagate2 with D (anti-symmetric), f = -A_x/2
//   x2: P_x2 P_x1^H, cn_hm_propagate1 with 1/r, f = +A_x/2
//   y1: P_y1 P_x2^H, propagate2 with D, f = -A_y/2
//   y2: P_y2 P_y1^H, propagate1 with 1/r, f = -A_y/2, then P_y2^H
// then the field-free step and the mirror image with the t_f values.  Component steps are
// dt/2 (cn_1e.hpp:869-872); propagate1 uses ifet = i lam f step/2, propagate2 ifet = -lam f
// step/2 (propagate.hpp:443-568).
struct oracle_vgwr {
	int32_t n_r, p, n_l, n_m, m0, n_inst;
	double dt;
	const double* S;      // [n_r][p+1]
	const double* Rinv;   // [n_r][p+1]  <B|1/r|B>
	const double* D;      // [n_r][p+1]  <B_i|d/dr B_j>, upper entries of an anti-symmetric band
	const double* upper;  // [lmax+1][n_r][p+1] complex, S - i dt/2 H_l
	const double* lower;  // [lmax+1][n_r][p+1] complex, lu_zsb(S + i dt/2 H_l)
	const double* lam[4]; // [N_ch] eigenvalues of x1, x2, y1, y2
	const double* P[4];   // [N_ch][N_ch] complex, P Z P^H = diag(lam)
};

// dst[k][r] = sum_ch A[k][ch] src[ch][r] (A complex N x N, conj_t: use A^H)
static void dense_apply(int N, int nr, const cx* A, bool herm, const cx* src, cx* dst)
{
	for (int k = 0; k < N; ++k)
		for (int r = 0; r < nr; ++r) dst[(long)k * nr + r] = {0.0, 0.0};
	for (int k = 0; k < N; ++k)
		for (int c = 0; c < N; ++c) {
			cx a = herm ? cx{A[(long)c * N + k].re, -A[(long)c * N + k].im} : A[(long)k * N + c];
			if (a.re == 0.0 && a.im == 0.0) continue;
			const cx* s = src + (long)c * nr;
			cx* d = dst + (long)k * nr;
			for (int r = 0; r < nr; ++r) d[r] = cadd(d[r], cmul(a, s[r]));
		}
}

static std::vector<cx> merge(int N, const cx* L, const cx* R)
{	// L R^H
	std::vector<cx> M((size_t)N * N, cx{0.0, 0.0});
	for (int i = 0; i < N; ++i)
		for (int j = 0; j < N; ++j) {
			cx s = {0.0, 0.0};
			for (int k = 0; k < N; ++k) s = cadd(s, cmul(L[(long)i * N + k], cx{R[(long)j * N + k].re, -R[(long)j * N + k].im}));
			M[(size_t)i * N + j] = s;
		}
	return M;
}

static void vg_component(const oracle_vgwr* g, cx* w, int comp, double f, std::vector<cx>& y, std::vector<cx>& u)
{
	const int N = g->n_l * g->n_m, nr = g->n_r, p = g->p;
	const double step = g->dt * 0.5;
	const bool anti = comp == 0 || comp == 2;
	const double frdt = f * step;
	for (int c = 0; c < N; ++c) {
		double lam = g->lam[comp][c];
		cx ifet = anti ? cx{lam * (-frdt / 2), 0.0} : cx{lam * 0.0, lam * (frdt / 2)};
		cn_channel(nr, p, g->S, anti ? g->D : g->Rinv, ifet, w + (long)c * nr, y.data(), u.data(), anti);
	}
}

void oracle_vgwr_step(const oracle_vgwr* g, double* coef, const double* ax_ti, const double* ax_tf, const double* ay_ti,
	const double* ay_tf, int nthreads)
{
	const int N = g->n_l * g->n_m, nr = g->n_r, p = g->p;
	const long per = (long)N * nr;
	const cx* P[4] = {(const cx*)g->P[0], (const cx*)g->P[1], (const cx*)g->P[2], (const cx*)g->P[3]};
	std::vector<cx> m12 = merge(N, P[1], P[0]), m23 = merge(N, P[2], P[1]), m34 = merge(N, P[3], P[2]);
	#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
	for (int k = 0; k < g->n_inst; ++k) {
		cx* c = (cx*)coef + k * per;
		std::vector<cx> w(per), y(nr), u((size_t)nr * p), wk(nr);
		if (!ax_ti) {
			for (int im = 0; im < g->n_m; ++im)
				for (int il = 0; il < g->n_l; ++il) {
					long l = lof(im, il, g->m0);
					cx* z = c + ((long)im * g->n_l + il) * nr;
					hc_channel(nr, p, (const cx*)g->upper + l * nr * (p + 1), (const cx*)g->lower + l * nr * (p + 1), z, wk.data());
				}
			continue;
		}
		const double axi = ax_ti[k] / 2.0, axf = ax_tf[k] / 2.0, ayi = ay_ti[k] / 2.0, ayf = ay_tf[k] / 2.0;
		dense_apply(N, nr, P[0], false, c, w.data());
		vg_component(g, w.data(), 0, -axi, y, u);
		dense_apply(N, nr, m12.data(), false, w.data(), c);
		vg_component(g, c, 1, axi, y, u);
		dense_apply(N, nr, m23.data(), false, c, w.data());
		vg_component(g, w.data(), 2, -ayi, y, u);
		dense_apply(N, nr, m34.data(), false, w.data(), c);
		vg_component(g, c, 3, -ayi, y, u);
		dense_apply(N, nr, P[3], true, c, w.data());
		for (int im = 0; im < g->n_m; ++im)
			for (int il = 0; il < g->n_l; ++il) {
				long l = lof(im, il, g->m0);
				cx* z = w.data() + ((long)im * g->n_l + il) * nr;
				hc_channel(nr, p, (const cx*)g->upper + l * nr * (p + 1), (const cx*)g->lower + l * nr * (p + 1), z, wk.data());
			}
		dense_apply(N, nr, P[3], false, w.data(), c);
		vg_component(g, c, 3, -ayf, y, u);
		dense_apply(N, nr, m34.data(), true, c, w.data());
		vg_component(g, w.data(), 2, -ayf, y, u);
		dense_apply(N, nr, m23.data(), true, w.data(), c);
		vg_component(g, c, 1, axf, y, u);
		dense_apply(N, nr, m12.data(), true, c, w.data());
		vg_component(g, w.data(), 0, -axf, y, u);
		dense_apply(N, nr, P[0], true, w.data(), c);
	}
}

// nt_total steps per instance: step s < nt_field uses (A_x, A_y) at t_s and t_{s+1} from
// atab[(inst*ld + s)*2 + {0,1}], later steps are field-free
void oracle_vgwr_run(const oracle_vgwr* g, double* coef, const double* atab, long ld, const int64_t* nt_field,
	const int64_t* nt_total, int nthreads)
{
	const long per = (long)g->n_l * g->n_m * g->n_r;
	#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
	for (int k = 0; k < g->n_inst; ++k) {
		oracle_vgwr one = *g;
		one.n_inst = 1;
		double* c = coef + 2 * k * per;
		for (long s = 0; s < nt_total[k]; ++s) {
			if (s < nt_field[k]) {
				const double* a = atab + (k * ld + s) * 2;
				oracle_vgwr_step(&one, c, a, a + 2, a + 1, a + 3, 1);
			} else oracle_vgwr_step(&one, c, nullptr, nullptr, nullptr, nullptr, 1);
		}
	}
}

} // extern "C"
