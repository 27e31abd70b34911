// GB300 (sm_103a) engine for the QPC-TDSE velocity-gauge elliptical Crank-Nicolson step,
// propagator_cn_hc_vgwr (spherical/propagator/cn_1e.hpp:812-951).
//
// One step with vector potential (A_x, A_y) is, with a = A/2 (cn_1e.hpp:911-914),
//   C_x1(-a_x) C_x2(a_x) C_y1(-a_y) C_y2(-a_y)  F  C_y2(-a_y') C_y1(-a_y') C_x2(a_x') C_x1(-a_x')
// (the mirror half with the t_f values), where each coupling C_c(f) = P_c^H M_c(f) P_c is a
// dense (m,l) transform to the eigenbasis of the angular operator Z_c (Y11 or Q11 times
// 1 or -i) and one banded CN per eigen-channel:
//   M(f) = (S + ifet O)^-1 (S - ifet O),  O = 1/r (symmetric, ifet = i lam f dt/8) for x2, y2,
//                                          O = d/dr (anti-symmetric, ifet = -lam f dt/8) for x1, y1
// (cn_hm_propagate1/2, propagate.hpp:443-568; component step dt/2), and consecutive
// transforms are merged, P_x2 P_x1^H etc. (cn_1e.hpp:884-889).  F is the field-free CN of
// every (m,l) channel.
//
// GB300 mapping: Z couples (m, l) only to (m +- 1, l +- 1), so it keeps il mod 2 (two parity
// blocks) and, inside a block, pairs the im-even with the im-odd channels only: Z = [[0, C], [C^T, 0]].
// The SVD of C gives its eigenvectors in pairs (u, +-v)/sqrt 2, so a transform is two real GEMMs of
// half the size (U on one m-parity set, V on the other) and an elementwise pairing step, and each
// backward transform merges with the next forward one into one pair of real GEMMs: per step 10
// transforms of 2 n^2 N flops each (n = block size) instead of the reference's dense complex
// N_ch x N_ch products.  The GEMMs are this library's own FP64 kernels (qpc_gemm.cuh), over the
// live wavefunctions; the SVDs come from cuSOLVER gesvd at set-up.  The banded CN of each
// eigen-channel runs one chain per thread as z := 2 (S + ifet O)^-1 S z - z: a real LU for the
// d/dr components (ifet real), an LU that uses the symmetry of S + ifet/r for the 1/r components,
// formed row by row with the previous p rows of U in registers and the forward substitution fused,
// U rows kept in a scratch buffer for the backward substitution.
// The field-free step uses the LDL^T factors of S + i dt/2 H_l (qpc_ldlt_csym) as
// x = 2 (S + i dt/2 H)^-1 S c - c.  State layout [inst][m][l][r] complex128, the
// reference's own.  All arithmetic is complex FP64.
#include "qpc_internal.h"
#include "qpc_cuda_util.cuh"
#include <cuda_runtime.h>
#include <cusolverDn.h>
#include "qpc_gemm.cuh"
#include "qpc_ozaki.cuh"
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <vector>
#include <algorithm>
#include <numeric>

namespace qpc {
namespace {

constexpr int VG_THREADS = 64;

__device__ __forceinline__ double2 cmul(double2 x, double2 y)
{
	return make_double2(fma(y.x, x.x, -(y.y * x.y)), fma(y.x, x.y, y.y * x.x));
}
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 crcp(double2 y)
{
	double d = fma(y.x, y.x, y.y * y.y);
	return make_double2(y.x / d, -y.y / d);
}

// One coupling component on the live prefix of instances: z := (S + e O)^-1 (S - e O) z per
// (instance, eigen-channel), computed as z := 2 (S + e O)^-1 S z - z (S - e O = 2 S - (S + e O)),
// so the right-hand side is the real band S times z.  e = lam[ch] * coef * f_inst with
// f_inst = sgn * A[(inst*ld + step + tofs)*2 + axis] / 2.  A channel with e = 0 has M = I and is
// left as it is.  One chain per thread: the factorisation is formed row by row with the previous
// P rows of U in registers (diagonal kept as its reciprocal) and the forward substitution fused;
// the U rows and y go to a scratch array for the backward pass, laid out element-major over the
// threads ((row * elements + e) * threads + t) so that a warp's stores and loads are contiguous.

// anti-symmetric O (d/dr: O(r, r+c) = band[r][c], O(r+c, r) = -band[r][c], c > 0) with e real
// (x1, y1): A = S + e O is a real non-symmetric band, factorised by a real LU without pivoting.  Each
// chain runs on a lane pair: the factor is real, so the real (part 0) and imaginary (part 1) parts of
// the solve are independent; both lanes form the same LU and each solves its own part.  Scratch (doubles) per row: U(i, i+1..i+P), 1/U(i, i) (written by part 0), y real, y imaginary,
// element e of row i of chain t at (i NSA + e) nth + t, NSA = P + 3.
template <int P>
__global__ void __launch_bounds__(VG_THREADS) k_vg_cn_anti2(double2* __restrict__ state, double* __restrict__ scr, const double* __restrict__ S,
	const double* __restrict__ O, const double* __restrict__ lam, double cre, const double* __restrict__ atab, long ld, long step, int tofs,
	int axis, double sgn, const int* __restrict__ perm, int N, int nch, int nlive)
{
	const long nth = (long)nlive * nch;
	const long tt = (long)blockIdx.x * VG_THREADS + threadIdx.x;
	const long t = tt >> 1;
	const int part = (int)(tt & 1);
	if (t >= nth) return;
	const int k = (int)(t / nch), ch = (int)(t - (long)k * nch);
	const double f = sgn * atab[((long)perm[k] * ld + step + tofs) * 2 + axis] / 2.0;
	const double e = lam[ch] * f * cre;
	if (e == 0.0) return;
	constexpr int NE = P + 1, NS = P + 3;
	double* z = reinterpret_cast<double*>(state + t * N) + part;	// own part, stride 2
	double Uw[P][NE];	// slot q: row i-1-q, [0] = 1/U(row, row), [c] = U(row, row + c)
	double yw[P], zw[P];	// own parts of y and z of the previous P rows
#pragma unroll
	for (int q = 0; q < P; ++q) {
		yw[q] = zw[q] = 0.0;
#pragma unroll
		for (int c = 0; c < NE; ++c) Uw[q][c] = 0.0;
	}
	for (int i = 0; i < N; ++i) {
		double lo[P], up[NE];
		double w = 0.0;
#pragma unroll
		for (int q = 0; q < P; ++q) {
			lo[q] = 0.0;
			if (i - 1 - q >= 0) {
				const double sv = S[(long)(i - 1 - q) * NE + q + 1], ov = O[(long)(i - 1 - q) * NE + q + 1];
				lo[q] = fma(-e, ov, sv);
				w = fma(sv, zw[q], w);
			}
		}
		const double zi = z[2L * i];
#pragma unroll
		for (int c = 0; c < NE; ++c) {
			up[c] = 0.0;
			if (i + c < N) {
				const double sv = S[(long)i * NE + c], ov = O[(long)i * NE + c];
				up[c] = fma(e, ov, sv);
				w = fma(sv, c ? z[2L * (i + c)] : zi, w);
			}
		}
		double l[P];
#pragma unroll
		for (int qq = P - 1; qq >= 0; --qq) {
			l[qq] = lo[qq] * Uw[qq][0];
#pragma unroll
			for (int c = 1; c < NE; ++c) {
				const int dc = c - 1 - qq;
				if (dc < 0) lo[-dc - 1] = fma(-l[qq], Uw[qq][c], lo[-dc - 1]);
				else up[dc] = fma(-l[qq], Uw[qq][c], up[dc]);
			}
		}
		double y = w;
#pragma unroll
		for (int q = 0; q < P; ++q) y = fma(-l[q], yw[q], y);
		const double ri = 1.0 / up[0];
		double* sr = scr + (long)i * NS * nth + t;
		if (part == 0) {
#pragma unroll
			for (int c = 1; c < NE; ++c) sr[(c - 1) * nth] = up[c];
			sr[P * nth] = ri;
		}
		sr[(P + 1 + part) * nth] = y;
#pragma unroll
		for (int q = P - 1; q > 0; --q) {
			yw[q] = yw[q - 1];
			zw[q] = zw[q - 1];
#pragma unroll
			for (int c = 0; c < NE; ++c) Uw[q][c] = Uw[q - 1][c];
		}
		yw[0] = y;
		zw[0] = zi;
		Uw[0][0] = ri;
#pragma unroll
		for (int c = 1; c < NE; ++c) Uw[0][c] = up[c];
	}
	// the U rows part 0 wrote are read by both lanes: order the pair's memory accesses
	__syncwarp(3u << (threadIdx.x & 30));
	double xw[P];
#pragma unroll
	for (int q = 0; q < P; ++q) xw[q] = 0.0;
	for (int i = N - 1; i >= 0; --i) {
		const double* sr = scr + (long)i * NS * nth + t;
		double v = sr[(P + 1 + part) * nth];
#pragma unroll
		for (int c = 1; c < NE; ++c) v = fma(-sr[(c - 1) * nth], xw[c - 1], v);
		const double x = v * sr[P * nth];
#pragma unroll
		for (int q = P - 1; q > 0; --q) xw[q] = xw[q - 1];
		xw[0] = x;
		const double zi = z[2L * i];
		z[2L * i] = fma(2.0, x, -zi);
	}
}

// symmetric O (1/r) with e = i b imaginary (x2, y2): A = S + i b O is complex symmetric, so in the
// row-by-row LU the multipliers of row i are U(col, i) / U(col, col) from the window (no elimination
// of the lower part) and only the upper part U(i, i..i+P) is formed.  Each chain runs on a lane pair:
// lane 2t + part holds part (0 real, 1 imaginary) of the chain's complex values and forms only its own
// part of every product (two FP64 instructions with operands chosen by integer selects), taking the
// partner's part by a shuffle within the pair.  The window of U rows is kept as own parts.  Scratch (doubles): part of element e of row i
// of chain t at ((i NS + e) nth + t) 2 + part, NS = P + 2.
__device__ __forceinline__ double pair_other(double v, unsigned pm) { return __shfl_xor_sync(pm, v, 1); }

// own part of a b from own (ao, bo) and partner (ae, be) parts: real ao bo - ae be, imaginary
// ae bo + ao be
__device__ __forceinline__ double own_mul(double ao, double ae, double bo, double be, int part)
{
	const double X = part ? ae : ao;
	const double Y = part ? ao : __longlong_as_double(__double_as_longlong(ae) ^ (long long)0x8000000000000000ull);
	return fma(X, bo, Y * be);
}
// acc - own part of a b
__device__ __forceinline__ double own_msub(double acc, double ao, double ae, double bo, double be, int part)
{
	const double X = part ? ae : ao;
	const double Y = part ? ao : __longlong_as_double(__double_as_longlong(ae) ^ (long long)0x8000000000000000ull);
	return fma(-X, bo, fma(-Y, be, acc));
}

template <int P>
__global__ void __launch_bounds__(VG_THREADS) k_vg_cn_sym2(double2* __restrict__ state, double* __restrict__ scr, const double* __restrict__ S,
	const double* __restrict__ O, const double* __restrict__ lam, double cim, const double* __restrict__ atab, long ld, long step, int tofs,
	int axis, double sgn, const int* __restrict__ perm, int N, int nch, int nlive)
{
	const long nth = (long)nlive * nch;
	const long tt = (long)blockIdx.x * VG_THREADS + threadIdx.x;
	const long t = tt >> 1;
	const int part = (int)(tt & 1);
	const unsigned pm = 3u << (threadIdx.x & 30);	// the lane pair of this chain
	if (t >= nth) return;	// both lanes of a pair leave together
	const int k = (int)(t / nch), ch = (int)(t - (long)k * nch);
	const double f = sgn * atab[((long)perm[k] * ld + step + tofs) * 2 + axis] / 2.0;
	const double b = lam[ch] * f * cim;
	if (b == 0.0) return;	// both lanes: the same chain
	constexpr int NE = P + 1, NS = P + 2;
	double* z = reinterpret_cast<double*>(state + t * N) + part;	// own part, stride 2
	double Uw[P][NE];	// own parts: slot q = row i-1-q, [0] = 1/U(row, row), [c] = U(row, row + c)
	double yw[P], yo[P], zw[P];	// y own / partner parts, z own part of the previous P rows
#pragma unroll
	for (int q = 0; q < P; ++q) {
		yw[q] = yo[q] = zw[q] = 0.0;
#pragma unroll
		for (int c = 0; c < NE; ++c) Uw[q][c] = 0.0;
	}
	for (int i = 0; i < N; ++i) {
		double w = 0.0;	// own part of (S z)_i
#pragma unroll
		for (int q = 0; q < P; ++q)
			if (i - 1 - q >= 0) w = fma(S[(long)(i - 1 - q) * NE + q + 1], zw[q], w);
		const double zi = z[2L * i];
		double up[NE];	// own parts of A(i, i+c) = S + i b O
#pragma unroll
		for (int c = 0; c < NE; ++c) {
			up[c] = 0.0;
			if (i + c < N) {
				const double sv = S[(long)i * NE + c];
				up[c] = part ? b * O[(long)i * NE + c] : sv;
				w = fma(sv, c ? z[2L * (i + c)] : zi, w);
			}
		}
		// multipliers L(i, i-1-q) = U(i-1-q, i) / U(i-1-q, i-1-q), both parts
		double lo[P], le[P];
#pragma unroll
		for (int q = 0; q < P; ++q) {
			const double uo = Uw[q][q + 1], ue = pair_other(uo, pm);
			const double ro = Uw[q][0], re = pair_other(ro, pm);
			lo[q] = own_mul(uo, ue, ro, re, part);
			le[q] = pair_other(lo[q], pm);
		}
		// U(i, i+c) = A(i, i+c) - sum_q L(i, i-1-q) U(i-1-q, i+c)
#pragma unroll
		for (int c = 0; c < P; ++c)
#pragma unroll
			for (int q = 0; q + c + 1 <= P; ++q) {
				const double uo = Uw[q][c + 1 + q], ue = pair_other(uo, pm);
				up[c] = own_msub(up[c], lo[q], le[q], uo, ue, part);
			}
		double y = w;
#pragma unroll
		for (int q = 0; q < P; ++q) y = own_msub(y, lo[q], le[q], yw[q], yo[q], part);
		// 1 / U(i, i): |U|^2 from both parts, own part of the conjugate over it
		const double u0e = pair_other(up[0], pm);
		const double d = fma(up[0], up[0], u0e * u0e);
		const double rinv = 1.0 / d;
		const double ri = part ? -up[0] * rinv : up[0] * rinv;
		double* sr = scr + ((long)i * NS * nth + t) * 2 + part;
#pragma unroll
		for (int c = 1; c < NE; ++c) sr[(long)(c - 1) * nth * 2] = up[c];
		sr[(long)P * nth * 2] = ri;
		sr[(long)(P + 1) * nth * 2] = y;
		const double ye = pair_other(y, pm);
#pragma unroll
		for (int q = P - 1; q > 0; --q) {
			yw[q] = yw[q - 1];
			yo[q] = yo[q - 1];
			zw[q] = zw[q - 1];
#pragma unroll
			for (int c = 0; c < NE; ++c) Uw[q][c] = Uw[q - 1][c];
		}
		yw[0] = y;
		yo[0] = ye;
		zw[0] = zi;
		Uw[0][0] = ri;
#pragma unroll
		for (int c = 1; c < NE; ++c) Uw[0][c] = up[c];
	}
	// backward: x_i = (y_i - sum_c U(i, i+c) x_{i+c}) / U(i, i); z_i := 2 x_i - z_i
	double xw[P], xe[P];
#pragma unroll
	for (int q = 0; q < P; ++q) xw[q] = xe[q] = 0.0;
	for (int i = N - 1; i >= 0; --i) {
		const double* sr = scr + ((long)i * NS * nth + t) * 2 + part;
		double v = sr[(long)(P + 1) * nth * 2];
#pragma unroll
		for (int c = 1; c < NE; ++c) {
			const double uo = sr[(long)(c - 1) * nth * 2], ue = pair_other(uo, pm);
			v = own_msub(v, uo, ue, xw[c - 1], xe[c - 1], part);
		}
		const double ro = sr[(long)P * nth * 2], re = pair_other(ro, pm);
		const double ve = pair_other(v, pm);
		const double x = own_mul(v, ve, ro, re, part);
		const double xo = pair_other(x, pm);
#pragma unroll
		for (int q = P - 1; q > 0; --q) { xw[q] = xw[q - 1]; xe[q] = xe[q - 1]; }
		xw[0] = x;
		xe[0] = xo;
		const double zi = z[2L * i];
		z[2L * i] = fma(2.0, x, -zi);
	}
}

// field-free step of every (instance, m, l) channel whose instance is still running:
// x = 2 (S + i dt/2 H_l)^-1 S c - c with the LDL^T factors Lrow[l][r][k-1] = L(r, r-k),
// Dinv[l][r] (qpc_ldlt_csym); y kept in the scratch buffer
template <int P>
__global__ void __launch_bounds__(VG_THREADS) k_vg_ff(double2* __restrict__ state, double2* __restrict__ ybuf, const double* __restrict__ S,
	const double2* __restrict__ Lrow, const double2* __restrict__ Dinv, const long long* __restrict__ ntt, const int* __restrict__ perm,
	const int* __restrict__ chmap, long step, int N, int nl, int nm, int m0, int nlh, int B)
{
	const long t = (long)blockIdx.x * VG_THREADS + threadIdx.x;
	const int nch = nl * nm;
	if (t >= (long)B * nch) return;
	const int k = (int)(t / nch), ch = (int)(t - (long)k * nch);
	if (step >= ntt[perm[k]]) return;
	const int och = chmap[ch];
	const int im = och / nl, il = och - im * nl;
	const int l = il + abs(m0 + im);
	constexpr int NE = P + 1;
	double2* c = state + t * N;
	double2* y = ybuf + t * N;
	const double2* L = Lrow + (long)l * N * P;
	const double2* Di = Dinv + (long)l * N;
	double2 w[P];
#pragma unroll
	for (int q = 0; q < P; ++q) w[q] = make_double2(0.0, 0.0);
	for (int i = 0; i < N; ++i) {
		double2 s = make_double2(0.0, 0.0);
#pragma unroll
		for (int j = 1; j <= P; ++j)
			if (i - j >= 0) { double b = S[(long)(i - j) * NE + j]; double2 v = c[i - j]; s.x = fma(b, v.x, s.x); s.y = fma(b, v.y, s.y); }
#pragma unroll
		for (int j = 0; j <= P; ++j)
			if (i + j < N) { double b = S[(long)i * NE + j]; double2 v = c[i + j]; s.x = fma(b, v.x, s.x); s.y = fma(b, v.y, s.y); }
#pragma unroll
		for (int q = 0; q < P; ++q) s = csub(s, cmul(L[(long)i * P + q], w[q]));
#pragma unroll
		for (int q = P - 1; q > 0; --q) w[q] = w[q - 1];
		w[0] = s;
		y[i] = cmul(s, Di[i]);
	}
#pragma unroll
	for (int q = 0; q < P; ++q) w[q] = make_double2(0.0, 0.0);
	for (int i = N - 1; i >= 0; --i) {
		double2 x = y[i];
#pragma unroll
		for (int q = 0; q < P; ++q)
			if (i + 1 + q < N) x = csub(x, cmul(L[(long)(i + 1 + q) * P + q], w[q]));
#pragma unroll
		for (int q = P - 1; q > 0; --q) w[q] = w[q - 1];
		w[0] = x;
		double2 ci = c[i];
		c[i] = make_double2(2.0 * x.x - ci.x, 2.0 * x.y - ci.y);
	}
}

// out[i][k] = in[i + k n]: a column-major n x n matrix (as cuSOLVER returns it) to row-major
__global__ void k_vg_transpose(const double* __restrict__ in, int n, double* __restrict__ out)
{
	const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= (long)n * n) return;
	const int i = (int)(t / n), k = (int)(t - (long)i * n);
	out[t] = in[(long)k * n + i];
}

// out[i][k] = s[i] in[i][k] (row-major n x n)
__global__ void k_vg_scale_rows(const double* __restrict__ in, const double* __restrict__ sg, int n, double* __restrict__ out)
{
	const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= (long)n * n) return;
	out[t] = sg[t / n] * in[t];
}

// The parity blocks of a transform in the engine's order: block b spans channels off[b] ..
// off[b] + na[b] + ns[b]; its larger m-parity set (na[b] channels) comes first, then the smaller
// one (ns[b]).  Eigen-channel order in a block: k+ (k < ns), the null channels (ns <= k < na),
// k- (row na + k, k < ns).
struct vg_blocks {
	int off[2], na[2], ns[2];
};

// The pairing step of a transform, in place on the live instances of X: forward
// w(k+-) = (gA a_k +- gB b_k)/sqrt 2 and w(null k) = gA a_k after the GEMMs a = U^T z_A, b = V^T z_B;
// inverse a'_k = conj(gA) (w(k+) + w(k-))/sqrt 2, b'_k = conj(gB) (w(k+) - w(k-))/sqrt 2,
// a'(null k) = conj(gA) w(null k) before the GEMMs z_A = U a', z_B = V b'.  g = the common phase of a
// set under the component's phase matrix (1, or -i for the im-odd set).
__global__ void k_vg_butterfly(double2* __restrict__ X, vg_blocks bk, int N, int nch, int nlive, int inv, double2 g0A, double2 g0B,
	double2 g1A, double2 g1B)
{
	const long per = (long)(bk.na[0] + bk.na[1]) * N;
	const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= (long)nlive * per) return;
	const long inst = t / per, e = t - inst * per;
	const int row = (int)(e / N), r = (int)(e - (long)row * N);
	const int b = row < bk.na[0] ? 0 : 1;
	const int k = b ? row - bk.na[0] : row;
	const double2 gA = b ? g1A : g0A, gB = b ? g1B : g0B;
	double2* base = X + (inst * nch + bk.off[b]) * (long)N + r;
	double2* pa = base + (long)k * N;
	const double h = 0.70710678118654752440;
	if (k < bk.ns[b]) {
		double2* pb = base + (long)(bk.na[b] + k) * N;
		const double2 a = *pa, c = *pb;
		if (!inv) {
			const double2 x = cmul(gA, a), y = cmul(gB, c);
			*pa = make_double2((x.x + y.x) * h, (x.y + y.y) * h);
			*pb = make_double2((x.x - y.x) * h, (x.y - y.y) * h);
		} else {
			const double2 sm = make_double2((a.x + c.x) * h, (a.y + c.y) * h), df = make_double2((a.x - c.x) * h, (a.y - c.y) * h);
			*pa = cmul(make_double2(gA.x, -gA.y), sm);
			*pb = cmul(make_double2(gB.x, -gB.y), df);
		}
	} else {
		*pa = inv ? cmul(make_double2(gA.x, -gA.y), *pa) : cmul(gA, *pa);
	}
}

// engine channel order (il-even channels first) <-> the reference's [m][l] order
__global__ void k_vg_permute(const double2* __restrict__ src, double2* __restrict__ dst, const int* __restrict__ chmap, int N, int nch,
	long total, bool to_engine)
{
	const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= total) return;
	const long per = (long)nch * N;
	const long k = i / per, e = i - k * per;
	const int t = (int)(e / N), r = (int)(e - (long)t * N);
	const long o = k * per + (long)chmap[t] * N + r;
	if (to_engine) dst[i] = src[o];
	else dst[o] = src[i];
}

// In-loop dipole of the elliptical driver (observable_r, spherical/observable/1e.hpp:52-129, recorded
// before every step at binsrc/sphTDSE.cpp:515-527): rm = sum over the channel pairs (m, l) -> (m+1, l +- 1)
// of coef * <c_{m,l}| F |c_{m+1,l+-1}> with F = <B|f(r)|B> (f = r) and the sin(theta) e^{-i phi} elements
// (integrate_sinexp1/2); x = Re rm, y = -Im rm (rp = conj(rm): the +1 elements are the transposed -1
// ones).  Partial sums per block over a contiguous range of (pair, row) items of one instance, then a
// fixed-order sum per instance: deterministic.
constexpr int DIP_THREADS = 256;
__global__ void __launch_bounds__(DIP_THREADS) k_vg_dip_part(const double2* __restrict__ state, const double* __restrict__ F,
	const int2* __restrict__ pairs, const double* __restrict__ pcoef, int npairs, int N, int P, int nch,
	const long long* __restrict__ ntt, const int* __restrict__ perm, long step, double2* __restrict__ part)
{
	const int k = blockIdx.y;	// instance slot (sorted order)
	const int nblk = gridDim.x;
	double2 acc = make_double2(0.0, 0.0);
	if (step < ntt[perm[k]]) {
		const long items = (long)npairs * N;
		const long per = (items + nblk - 1) / nblk;
		const long i0 = (long)blockIdx.x * per, i1 = min(items, i0 + per);
		const double2* x = state + (long)k * nch * N;
		for (long it = i0 + threadIdx.x; it < i1; it += DIP_THREADS) {
			const int pr = (int)(it / N), r = (int)(it - (long)pr * N);
			const int2 ab = pairs[pr];
			const double2* ca = x + (long)ab.x * N;
			const double2* cb = x + (long)ab.y * N;
			double tr = 0.0, ti = 0.0;	// (F c_b)(r)
			for (int q = 1; q <= P && q <= r; ++q) { const double f = F[(long)(r - q) * (P + 1) + q]; const double2 v = cb[r - q]; tr = fma(f, v.x, tr); ti = fma(f, v.y, ti); }
			for (int q = 0; q <= P && r + q < N; ++q) { const double f = F[(long)r * (P + 1) + q]; const double2 v = cb[r + q]; tr = fma(f, v.x, tr); ti = fma(f, v.y, ti); }
			const double2 a = ca[r];
			const double c = pcoef[pr];
			// conj(a) * t * c
			acc.x = fma(c, fma(a.x, tr, a.y * ti), acc.x);
			acc.y = fma(c, fma(a.x, ti, -(a.y * tr)), acc.y);
		}
	}
	__shared__ double2 sm[DIP_THREADS];
	sm[threadIdx.x] = acc;
	__syncthreads();
	for (int w = DIP_THREADS / 2; w > 0; w >>= 1) {
		if ((int)threadIdx.x < w) { sm[threadIdx.x].x += sm[threadIdx.x + w].x; sm[threadIdx.x].y += sm[threadIdx.x + w].y; }
		__syncthreads();
	}
	if (threadIdx.x == 0) part[(long)k * nblk + blockIdx.x] = sm[0];
}

__global__ void k_vg_dip_final(const double2* __restrict__ part, int nblk, int nlive, const long long* __restrict__ ntt,
	const int* __restrict__ perm, long step, long ldz, double* __restrict__ xs, double* __restrict__ ys)
{
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= nlive || step >= ntt[perm[k]]) return;
	double2 rm = make_double2(0.0, 0.0);
	for (int b = 0; b < nblk; ++b) { rm.x += part[(long)k * nblk + b].x; rm.y += part[(long)k * nblk + b].y; }
	xs[(long)k * ldz + step] = rm.x;
	ys[(long)k * ldz + step] = -rm.y;
}

__global__ void k_vg_snorm(const double2* __restrict__ state, const double* __restrict__ S, int N, int P, int nch, double* out)
{
	// one block per instance, fixed-order reduction
	const int b = blockIdx.x;
	const double2* x = state + (long)b * nch * N;
	double acc = 0.0;
	for (long e = threadIdx.x; e < (long)nch * N; e += blockDim.x) {
		int r = (int)(e % N);
		double2 t = make_double2(0.0, 0.0);
		for (int q = 1; q <= P && q <= r; ++q) { double s = S[(long)(r - q) * (P + 1) + q]; double2 v = x[e - q]; t.x = fma(s, v.x, t.x); t.y = fma(s, v.y, t.y); }
		for (int q = 0; q <= P && r + q < N; ++q) { double s = S[(long)r * (P + 1) + q]; double2 v = x[e + q]; t.x = fma(s, v.x, t.x); t.y = fma(s, v.y, t.y); }
		acc = fma(x[e].x, t.x, fma(x[e].y, t.y, acc));
	}
	__shared__ double sm[256];
	sm[threadIdx.x] = acc;
	__syncthreads();
	for (int s = blockDim.x / 2; s > 0; s >>= 1) {
		if ((int)threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
		__syncthreads();
	}
	if (threadIdx.x == 0) out[b] = sm[0];
}

} // namespace
} // namespace qpc

using namespace qpc;

struct qpc_vgwr {
	int dev = 0;
	qpc_dims d{};
	int N = 0, P = 0, nch = 0, nlh = 0, B = 0;
	double dt = 0;
	cudaStream_t st = nullptr;
	cudaEvent_t ev0 = nullptr, ev1 = nullptr;
	double *S = nullptr, *Ri = nullptr, *D = nullptr;
	double *lam[4] = {nullptr, nullptr, nullptr, nullptr};
	// transforms, block-diagonal in the engine's channel order: block b (0: il even, 1: il odd)
	// spans nb[b] channels from off[b]; inside it the larger m-parity set (na[b] channels, im
	// parity apar[b]) comes first, then the smaller one (nb[b] - na[b])
	int nb[2] = {0, 0}, off[2] = {0, 0}, na[2] = {0, 0}, apar[2] = {0, 0};
	int* chmap = nullptr;                          // engine channel -> reference channel im*n_l+il
	// real transform matrices [mat][block][set] (row-major, set 0: na x na, set 1: ns x ns) in
	// tmbuf: mat 0 = U~_x1 (forward x1 = its transpose, backward = itself), 1 = U~_y2 (the same for
	// y2), 2 = M12 = U~_x2^T U~_x1, 3 = M23 = U~_y1^T U~_x2, 4 = M34 = U~_y2^T U~_y1 (merged backward
	// and forward transforms; their transposes run the mirror half)
	double* tmbuf = nullptr;
	double* tm[5][2][2] = {};
	double2 gam[4][2][2] = {};                    // [component][block][set]: the set's common phase
	// slice-product GEMM (qpc_ozaki.cuh): digit slices and exponent fields of every matrix per
	// orientation [mat][block][set][trans], and the scratch for the state's slices
	bool slices = true;
	__nv_bfloat16* sdA[5][2][2][2] = {};
	int* seA[5][2][2][2] = {};
	__nv_bfloat16* sdB = nullptr;
	int* seB = nullptr;
	double2 *Lrow = nullptr, *Dinv = nullptr;     // field-free factors
	double2 *X = nullptr, *W = nullptr;
	double2* U = nullptr;                          // CN scratch: (p + 2) complex per chain-row
	double* atab = nullptr;
	long atab_cap = 0;
	long long* ntt = nullptr;
	int* perm = nullptr;
	double* nrm = nullptr;
	float last_ms = 0.f;
	long launches = 0;
	// per-kernel timing (qpc_vgwr_set_profiling): events around each launch group,
	// summed per kind (0 transforms, 1 coupling CN, 2 field-free CN) after the run
	bool profiling = false;
	std::vector<cudaEvent_t> evpool;
	size_t evused = 0;
	struct mark { int kind; cudaEvent_t a, b; };
	std::vector<mark> marks;
	double kms[3] = {0, 0, 0};
	long kcnt[3] = {0, 0, 0};
	// in-loop dipole (qpc_vgwr_run_dipole): channel pairs in engine order, their coefficients,
	// the f(r) band, per-block partials and the recorded lists [B][ldz] in the sorted order
	int2* dpairs = nullptr;
	double* dcoef = nullptr;
	int ndpairs = 0;
	double* dF = nullptr;
	double2* dpart = nullptr;
	double *dxs = nullptr, *dys = nullptr;
	size_t dcap = 0;
	int dnblk = 1;
};

namespace {

void vg_free(qpc_vgwr* h)
{
	if (!h) return;
	cudaSetDevice(h->dev);
	void* ps[] = {h->S, h->Ri, h->D, h->lam[0], h->lam[1], h->lam[2], h->lam[3], h->tmbuf, h->Lrow,
		h->Dinv, h->X, h->W, h->U, h->atab, h->ntt, h->perm, h->nrm, h->chmap};
	for (void* p : ps) if (p) cudaFree(p);
	if (h->ev0) cudaEventDestroy(h->ev0);
	if (h->ev1) cudaEventDestroy(h->ev1);
	for (auto e : h->evpool) cudaEventDestroy(e);
	void* dp[] = {h->dpairs, h->dcoef, h->dF, h->dpart, h->dxs, h->dys, h->sdB, h->seB};
	for (void* p : dp) if (p) cudaFree(p);
	for (int m = 0; m < 5; ++m)
		for (int b = 0; b < 2; ++b)
			for (int st = 0; st < 2; ++st)
				for (int tr = 0; tr < 2; ++tr) {
					if (h->sdA[m][b][st][tr]) cudaFree(h->sdA[m][b][st][tr]);
					if (h->seA[m][b][st][tr]) cudaFree(h->seA[m][b][st][tr]);
				}
	if (h->st) cudaStreamDestroy(h->st);
	delete h;
}

// profiling marks: an event recorded before a launch group (begin) and after it (end)
cudaEvent_t pool_event(qpc_vgwr* h)
{
	if (h->evused == h->evpool.size()) {
		cudaEvent_t e = nullptr;
		if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
		h->evpool.push_back(e);
	}
	return h->evpool[h->evused++];
}
cudaEvent_t prof_begin(qpc_vgwr* h)
{
	if (!h->profiling) return nullptr;
	cudaEvent_t a = pool_event(h);
	if (a) cudaEventRecord(a, h->st);
	return a;
}
void prof_end(qpc_vgwr* h, int kind, cudaEvent_t a)
{
	if (!a) return;
	cudaEvent_t b = pool_event(h);
	if (!b) return;
	cudaEventRecord(b, h->st);
	h->marks.push_back({kind, a, b});
}
void prof_collect(qpc_vgwr* h)
{
	for (auto& m : h->marks) {
		float ms = 0.f;
		if (cudaEventElapsedTime(&ms, m.a, m.b) == cudaSuccess) { h->kms[m.kind] += ms; ++h->kcnt[m.kind]; }
	}
	h->marks.clear();
	h->evused = 0;
}

// the GEMM part of a transform: out rows of every set = op(matrix mat of the set) times the in rows
// of the same set, live instances, on the state viewed as [channel][2 N] reals (the matrices are
// real); trans: apply the transposes
void gemm_sets(qpc_vgwr* h, int mat, bool trans, const double2* in, double2* out, int nlive)
{
	const int N = h->N;
	const long sstate = (long)h->nch * N;
	for (int b = 0; b < 2; ++b)
		for (int st = 0; st < 2; ++st) {
			const int n = st ? h->nb[b] - h->na[b] : h->na[b];
			if (!n) continue;
			const long o = (long)(h->off[b] + (st ? h->na[b] : 0)) * N;
			if (h->slices) {
				// the state's rows of this set as the [n][2 N nlive] right operand: element (k, j) of
				// instance j / (2 N) at channel k, real j % (2 N); the product written back the same way
				const long J = 2L * N * nlive;
				oz_split(oz::operand{(const double*)(in + o), 2L * N, 1, 2 * sstate, 2L * N}, n, J, h->seB, h->sdB, h->st);
				oz_gemm(h->sdA[mat][b][st][trans ? 1 : 0], h->seA[mat][b][st][trans ? 1 : 0], h->sdB, h->seB, n, J, n, (double*)(out + o),
					2L * N, 2L * N, 2 * sstate, h->st);
				h->launches += 3;
				continue;
			}
			const dim3 g = gemm::grid_for(2 * N, n, nlive);
			const double* A = h->tm[mat][b][st];
			if (trans) gemm::k_dgemm<true><<<g, gemm::THREADS, 0, h->st>>>(A, n, (const double*)(in + o), (double*)(out + o), 2L * N, 2 * sstate, 2 * N);
			else gemm::k_dgemm<false><<<g, gemm::THREADS, 0, h->st>>>(A, n, (const double*)(in + o), (double*)(out + o), 2L * N, 2 * sstate, 2 * N);
			++h->launches;
		}
}

// the pairing step of component c's transform (forward or inverse) on X
void butterfly(qpc_vgwr* h, double2* X, int c, bool inv, int nlive)
{
	vg_blocks bk;
	for (int b = 0; b < 2; ++b) { bk.off[b] = h->off[b]; bk.na[b] = h->na[b]; bk.ns[b] = h->nb[b] - h->na[b]; }
	const long total = (long)nlive * (h->na[0] + h->na[1]) * h->N;
	if (total <= 0) return;
	k_vg_butterfly<<<(unsigned)((total + 255) / 256), 256, 0, h->st>>>(X, bk, h->N, h->nch, nlive, inv ? 1 : 0, h->gam[c][0][0],
		h->gam[c][0][1], h->gam[c][1][0], h->gam[c][1][1]);
	++h->launches;
}

// one transform between the l basis and the eigen-channels of components: forward to c1 (c0 < 0),
// backward from c0 (c1 < 0), or merged backward from c0 and forward to c1 with matrix mat
void transform(qpc_vgwr* h, int c0, int c1, int mat, bool trans, double2* in, double2* out, int nlive)
{
	cudaEvent_t pa = prof_begin(h);
	if (c0 >= 0) butterfly(h, in, c0, true, nlive);
	gemm_sets(h, mat, trans, in, out, nlive);
	if (c1 >= 0) butterfly(h, out, c1, false, nlive);
	prof_end(h, 0, pa);
}

template <int P>
int step_t(qpc_vgwr* h, long s, long ld, int nlive, int nff)
{
	// first half, live instances (prefix)
	const int nb = nlive;
	auto cn = [&](double2* z, int comp, int tofs) {
		const bool anti = comp == 0 || comp == 2;
		const double q = h->dt * 0.5 / 2.0;	// e = lam f (-q) for d/dr, i lam f q for 1/r
		const int axis = comp < 2 ? 0 : 1;
		const double sgn = comp == 1 ? 1.0 : -1.0;
		const long nth = (long)nb * h->nch;
		const unsigned grid = (unsigned)((nth + VG_THREADS - 1) / VG_THREADS);
		cudaEvent_t pa = prof_begin(h);
		if (anti)
			k_vg_cn_anti2<P><<<(unsigned)((2 * nth + VG_THREADS - 1) / VG_THREADS), VG_THREADS, 0, h->st>>>(z, (double*)h->U, h->S, h->D,
				h->lam[comp], -q, h->atab, ld, s, tofs, axis, sgn, h->perm, h->N, h->nch, nb);
		else
			k_vg_cn_sym2<P><<<(unsigned)((2 * nth + VG_THREADS - 1) / VG_THREADS), VG_THREADS, 0, h->st>>>(z, (double*)h->U, h->S, h->Ri,
				h->lam[comp], q, h->atab, ld, s, tofs, axis, sgn, h->perm, h->N, h->nch, nb);
		prof_end(h, 1, pa);
		++h->launches;
	};
	// components x1 (0), x2 (1), y1 (2), y2 (3); each backward transform is merged with the next
	// forward one (matrices M12, M23, M34, transposed in the mirror half)
	if (nb > 0) {
		transform(h, -1, 0, 0, true, h->X, h->W, nb);
		cn(h->W, 0, 0);
		transform(h, 0, 1, 2, false, h->W, h->X, nb);
		cn(h->X, 1, 0);
		transform(h, 1, 2, 3, false, h->X, h->W, nb);
		cn(h->W, 2, 0);
		transform(h, 2, 3, 4, false, h->W, h->X, nb);
		cn(h->X, 3, 0);
		transform(h, 3, -1, 1, false, h->X, h->W, nb);
		// W holds the live instances' states; the others are still in X
		QPC_CUDA(cudaMemcpyAsync(h->X, h->W, sizeof(double2) * (size_t)nb * h->nch * h->N, cudaMemcpyDeviceToDevice, h->st));
	}
	if (nff > 0) {
		const long nth = (long)nff * h->nch;
		cudaEvent_t pa = prof_begin(h);
		k_vg_ff<P><<<(unsigned)((nth + VG_THREADS - 1) / VG_THREADS), VG_THREADS, 0, h->st>>>(h->X, h->U, h->S, h->Lrow, h->Dinv, h->ntt,
			h->perm, h->chmap, s, h->N, h->d.n_l, h->d.n_m, h->d.m0, h->nlh, nff);
		prof_end(h, 2, pa);
		++h->launches;
	}
	if (nb > 0) {
		transform(h, -1, 3, 1, true, h->X, h->W, nb);
		cn(h->W, 3, 1);
		transform(h, 3, 2, 4, true, h->W, h->X, nb);
		cn(h->X, 2, 1);
		transform(h, 2, 1, 3, true, h->X, h->W, nb);
		cn(h->W, 1, 1);
		transform(h, 1, 0, 2, true, h->W, h->X, nb);
		cn(h->X, 0, 1);
		transform(h, 0, -1, 0, false, h->X, h->W, nb);
		QPC_CUDA(cudaMemcpyAsync(h->X, h->W, sizeof(double2) * (size_t)nb * h->nch * h->N, cudaMemcpyDeviceToDevice, h->st));
	}
	QPC_CUDA(cudaGetLastError());
	return QPC_OK;
}

int step_dispatch(qpc_vgwr* h, long s, long ld, int nlive, int nff)
{
	switch (h->P) {
	case 1: return step_t<1>(h, s, ld, nlive, nff);
	case 2: return step_t<2>(h, s, ld, nlive, nff);
	case 3: return step_t<3>(h, s, ld, nlive, nff);
	case 4: return step_t<4>(h, s, ld, nlive, nff);
	case 5: return step_t<5>(h, s, ld, nlive, nff);
	case 6: return step_t<6>(h, s, ld, nlive, nff);
	case 7: return step_t<7>(h, s, ld, nlive, nff);
	default: return step_t<8>(h, s, ld, nlive, nff);
	}
}

// reorder instance blocks: X[k] = X[perm[k]] (inverse: X[perm[k]] = X[k]) through W
int permute(qpc_vgwr* h, const std::vector<int>& perm, bool inverse)
{
	const size_t blk = sizeof(double2) * (size_t)h->nch * h->N;
	for (int k = 0; k < h->B; ++k) {
		int src = inverse ? k : perm[k], dst = inverse ? perm[k] : k;
		QPC_CUDA(cudaMemcpyAsync((char*)h->W + dst * blk, (char*)h->X + src * blk, blk, cudaMemcpyDeviceToDevice, h->st));
	}
	QPC_CUDA(cudaMemcpyAsync(h->X, h->W, blk * h->B, cudaMemcpyDeviceToDevice, h->st));
	return QPC_OK;
}

// Angular eigensystems on the device, block by block.  Z_c couples (m, l) only to (m +- 1, l +- 1):
// it keeps il mod 2 (the parity blocks) and flips the parity of im, so inside a block it pairs the
// im-even with the im-odd channels only: Z = [[0, C], [C^T, 0]] with C = Z[A, B] (A the larger
// m-parity set).  From the SVD C = U Sigma V^T its eigenvectors are (u_k, +-v_k)/sqrt 2 with
// eigenvalues +-sigma_k, and (u_k, 0) with eigenvalue 0 for the |A| - |B| left singular vectors
// beyond; so every transform is two real GEMMs of half the size (U on the A rows, V on the B rows)
// and a pairing step.  With D = diag(i^(m - m0)) the -i couplings are real symmetric,
// Z_R(y1) = -Z_R(x1) and Z_R(y2) = -Z_R(x2): one SVD per block and coupling type (Y11 for x1/y1,
// Q11 for x2/y2, cuSOLVER gesvd, set-up only) gives all four couplings (lam_y = -lam_x).  The
// phase (-i)^im that x2 and y1 carry is (-1)^(im/2) on im-even channels and -i (-1)^((im-1)/2) on
// im-odd ones: the signs go into the rows of U~ = diag(s) U, the common -i into the pairing step.
// Writes lam[c] in the engine's eigen order and the matrices tm.
int device_transforms(qpc_vgwr* h, std::vector<int>& chmap, std::vector<double> lam[4])
{
	const int nl = h->d.n_l, nm = h->d.n_m, N = h->nch;
	cusolverDnHandle_t sol = nullptr;
	if (cusolverDnCreate(&sol) != CUSOLVER_STATUS_SUCCESS) { set_error("cusolverDnCreate failed"); return QPC_ERR_CUDA; }
	struct guard { cusolverDnHandle_t s; std::vector<void*> p; ~guard() { for (void* q : p) if (q) cudaFree(q); if (s) cusolverDnDestroy(s); } } G{sol, {}};
	if (cusolverDnSetStream(sol, h->st) != CUSOLVER_STATUS_SUCCESS) { set_error("cusolverDnSetStream failed"); return QPC_ERR_CUDA; }
	auto scratch = [&](double** p, size_t n) -> int { int rc = dalloc(p, n); G.p.push_back(*p); return rc; };
	int rc;
	int* d_info = nullptr;
	if ((rc = dalloc(&d_info, 1))) return rc;
	G.p.push_back(d_info);
	for (int c = 0; c < 4; ++c) lam[c].assign(N, 0.0);
	// matrix storage: 5 matrices per block and set
	size_t tot = 0;
	for (int b = 0; b < 2; ++b) {
		const size_t a = (size_t)h->na[b], sn = (size_t)(h->nb[b] - h->na[b]);
		tot += 5 * (a * a + sn * sn);
	}
	if ((rc = dalloc(&h->tmbuf, std::max<size_t>(tot, 1)))) return rc;
	{
		size_t o = 0;
		for (int m = 0; m < 5; ++m)
			for (int b = 0; b < 2; ++b)
				for (int st = 0; st < 2; ++st) {
					const size_t n = st ? (size_t)(h->nb[b] - h->na[b]) : (size_t)h->na[b];
					h->tm[m][b][st] = h->tmbuf + o;
					o += n * n;
				}
	}
	// the base singular vectors U (set 0) / V (set 1) of Y11 (base 0) and Q11 (base 1), row-major
	// [i][k] = k-th singular vector's entry i, in scratch: ub[base][block][set]
	double* ub[2][2][2] = {};
	std::vector<double> Zr((size_t)N * N);
	for (int base = 0; base < 2; ++base) {
		vgwr_real_coupling(nl, nm, h->d.m0, base, Zr.data());
		const int cx = base == 0 ? 0 : 1, cy = base == 0 ? 2 : 3;
		for (int b = 0; b < 2; ++b) {
			const int na = h->na[b], ns = h->nb[b] - h->na[b], o = h->off[b];
			if ((rc = scratch(&ub[base][b][0], (size_t)std::max(na * na, 1))) || (rc = scratch(&ub[base][b][1], (size_t)std::max(ns * ns, 1))))
				return rc;
			if (!na) continue;
			if (!ns) {	// no partner set: Z is zero on the block, the transform is the identity
				std::vector<double> I((size_t)na * na, 0.0);
				for (int i = 0; i < na; ++i) I[(size_t)i * na + i] = 1.0;
				QPC_CUDA(cudaMemcpy(ub[base][b][0], I.data(), sizeof(double) * I.size(), cudaMemcpyHostToDevice));
				continue;
			}
			std::vector<double> Ccm((size_t)na * ns);	// column-major na x ns
			for (int j = 0; j < ns; ++j)
				for (int i = 0; i < na; ++i) Ccm[(size_t)j * na + i] = Zr[(size_t)chmap[o + i] * N + chmap[o + na + j]];
			double *A = nullptr, *Sg = nullptr, *Ucm = nullptr, *work = nullptr, *rwork = nullptr;
			if ((rc = scratch(&A, Ccm.size())) || (rc = scratch(&Sg, (size_t)ns)) || (rc = scratch(&Ucm, (size_t)na * na)) ||
				(rc = scratch(&rwork, (size_t)ns)))
				return rc;
			QPC_CUDA(cudaMemcpy(A, Ccm.data(), sizeof(double) * Ccm.size(), cudaMemcpyHostToDevice));
			int lwork = 0;
			if (cusolverDnDgesvd_bufferSize(sol, na, ns, &lwork) != CUSOLVER_STATUS_SUCCESS) { set_error("gesvd buffer size failed"); return QPC_ERR_CUDA; }
			if ((rc = scratch(&work, (size_t)std::max(lwork, 1)))) return rc;
			// VT (ns x ns, column-major) is V row-major: VT[k + j ns] = v_k[j] = V_rm[j][k]
			if (cusolverDnDgesvd(sol, 'A', 'A', na, ns, A, na, Sg, Ucm, na, ub[base][b][1], ns, work, lwork, rwork, d_info) != CUSOLVER_STATUS_SUCCESS) {
				set_error("gesvd failed"); return QPC_ERR_CUDA;
			}
			k_vg_transpose<<<(unsigned)(((long)na * na + 255) / 256), 256, 0, h->st>>>(Ucm, na, ub[base][b][0]);
			QPC_CUDA(cudaGetLastError());
			if ((rc = wait_on(h->st))) return rc;
			int info = 0;
			QPC_CUDA(cudaMemcpy(&info, d_info, sizeof(int), cudaMemcpyDeviceToHost));
			if (info) { set_error("gesvd info %d", info); return QPC_ERR_NUMERIC; }
			std::vector<double> sg(ns);
			QPC_CUDA(cudaMemcpy(sg.data(), Sg, sizeof(double) * ns, cudaMemcpyDeviceToHost));
			for (int k = 0; k < ns; ++k) {
				lam[cx][o + k] = sg[k];
				lam[cx][o + na + k] = -sg[k];
				lam[cy][o + k] = -sg[k];
				lam[cy][o + na + k] = sg[k];
			}
		}
	}
	// U~_c = diag(s) U for the components with the phase (x2, y1), U itself for x1, y2; merged
	// M12 = U~_x2^T U~_x1, M23 = U~_y1^T U~_x2, M34 = U~_y2^T U~_y1 per block and set
	for (int b = 0; b < 2; ++b)
		for (int st = 0; st < 2; ++st) {
			const int n = st ? h->nb[b] - h->na[b] : h->na[b];
			if (!n) continue;
			const int o = h->off[b] + (st ? h->na[b] : 0);
			std::vector<double> sgn(n);
			for (int i = 0; i < n; ++i) {
				const int im = chmap[o + i] / nl;
				sgn[i] = ((im & 1) ? ((im - 1) / 2) & 1 : (im / 2) & 1) ? -1.0 : 1.0;
			}
			double *ds = nullptr, *ux2 = nullptr, *uy1 = nullptr;
			if ((rc = scratch(&ds, (size_t)n)) || (rc = scratch(&ux2, (size_t)n * n)) || (rc = scratch(&uy1, (size_t)n * n))) return rc;
			QPC_CUDA(cudaMemcpy(ds, sgn.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
			const unsigned g = (unsigned)(((long)n * n + 255) / 256);
			QPC_CUDA(cudaMemcpyAsync(h->tm[0][b][st], ub[0][b][st], sizeof(double) * n * n, cudaMemcpyDeviceToDevice, h->st));
			QPC_CUDA(cudaMemcpyAsync(h->tm[1][b][st], ub[1][b][st], sizeof(double) * n * n, cudaMemcpyDeviceToDevice, h->st));
			k_vg_scale_rows<<<g, 256, 0, h->st>>>(ub[1][b][st], ds, n, ux2);
			k_vg_scale_rows<<<g, 256, 0, h->st>>>(ub[0][b][st], ds, n, uy1);
			const dim3 gg = gemm::grid_for(n, n, 1);
			gemm::k_dgemm<true><<<gg, gemm::THREADS, 0, h->st>>>(ux2, n, h->tm[0][b][st], h->tm[2][b][st], (long)n, 0L, n);
			gemm::k_dgemm<true><<<gg, gemm::THREADS, 0, h->st>>>(uy1, n, ux2, h->tm[3][b][st], (long)n, 0L, n);
			gemm::k_dgemm<true><<<gg, gemm::THREADS, 0, h->st>>>(h->tm[1][b][st], n, uy1, h->tm[4][b][st], (long)n, 0L, n);
			QPC_CUDA(cudaGetLastError());
			if ((rc = wait_on(h->st))) return rc;
		}
	// digit slices of every matrix in both orientations for the slice-product GEMM: op(A)(i, k) =
	// A[i n + k] (trans 0) or A[k n + i] (trans 1), rows of op(A) are the split's columns
	if (h->slices)
		for (int m = 0; m < 5; ++m)
			for (int b = 0; b < 2; ++b)
				for (int st = 0; st < 2; ++st) {
					const long n = st ? h->nb[b] - h->na[b] : h->na[b];
					if (!n) continue;
					for (int tr = 0; tr < 2; ++tr) {
						if ((rc = dalloc(&h->sdA[m][b][st][tr], oz_digits_elems(n, n))) || (rc = dalloc(&h->seA[m][b][st][tr], (size_t)n))) return rc;
						const oz::operand o = tr ? oz::operand{h->tm[m][b][st], n, 1, 0, n} : oz::operand{h->tm[m][b][st], 1, n, 0, n};
						if ((rc = oz_split(o, n, n, h->seA[m][b][st][tr], h->sdA[m][b][st][tr], h->st))) return rc;
					}
				}
	if ((rc = wait_on(h->st))) return rc;
	// the common phase of each set under each component: -i for an im-odd set of x2 and y1, else 1
	for (int c = 0; c < 4; ++c)
		for (int b = 0; b < 2; ++b)
			for (int st = 0; st < 2; ++st) {
				const int par = st ? 1 - h->apar[b] : h->apar[b];
				const bool phase = c == 1 || c == 2;
				h->gam[c][b][st] = (phase && par == 1) ? make_double2(0.0, -1.0) : make_double2(1.0, 0.0);
			}
	return QPC_OK;
}

} // namespace

extern "C" {

int qpc_vgwr_create(const qpc_dims* dims, double dt, const double* S, const double* Rinv, const double* D, const double* H,
	qpc_vgwr** out)
{
	if (!out) { set_error("out is NULL"); return QPC_ERR_ARGS; }
	*out = nullptr;
	if (!dims || !S || !Rinv || !D || !H) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	const qpc_dims d = *dims;
	if (d.p < 1 || d.p > QPC_MAX_RANK || d.n_r < 2 * d.p + 2 || d.n_l < 1 || d.n_m < 1 || d.n_inst < 1) {
		set_error("bad dims n_r=%d p=%d n_l=%d n_m=%d n_inst=%d", d.n_r, d.p, d.n_l, d.n_m, d.n_inst);
		return QPC_ERR_ARGS;
	}
	if (!(dt > 0) || !std::isfinite(dt)) { set_error("dt=%g", dt); return QPC_ERR_ARGS; }
	int dev = 0;
	if (int rc = check_device(&dev)) return rc;
	qpc_vgwr* h = new (std::nothrow) qpc_vgwr;
	if (!h) { set_error("host allocation"); return QPC_ERR_NOMEM; }
	auto fail = [&](int rc) { vg_free(h); return rc; };
	h->dev = dev; h->d = d; h->N = d.n_r; h->P = d.p; h->nch = d.n_l * d.n_m; h->B = d.n_inst; h->dt = dt;
	const int mmax = std::max(std::abs(d.m0), std::abs(d.m0 + d.n_m - 1));
	h->nlh = mmax + d.n_l;
	const int N = d.n_r, P = d.p, NE = P + 1, nch = h->nch;
	// field-free factors
	std::vector<double> lrow((size_t)h->nlh * N * P * 2), dinv((size_t)h->nlh * N * 2);
	for (int l = 0; l < h->nlh; ++l) {
		int bad = qpc_ldlt_csym(N, P, S, H + (size_t)l * N * NE, dt * 0.5, lrow.data() + (size_t)l * N * P * 2, dinv.data() + (size_t)l * N * 2);
		if (bad < 0) { set_error("ldlt arguments"); return fail(QPC_ERR_ARGS); }
		if (bad > 0) { set_error("zero pivot factorising S + i dt/2 H_%d", l); return fail(QPC_ERR_SINGULAR); }
	}
	if ((cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking)) != cudaSuccess) { set_error("cudaStreamCreateWithFlags failed"); return fail(QPC_ERR_CUDA); }
	if ((cudaEventCreate(&h->ev0)) != cudaSuccess) { set_error("cudaEventCreate failed"); return fail(QPC_ERR_CUDA); }
	if ((cudaEventCreate(&h->ev1)) != cudaSuccess) { set_error("cudaEventCreate failed"); return fail(QPC_ERR_CUDA); }
	const size_t nst = (size_t)h->B * nch * N;
	// engine channel order: the il-even block, then the il-odd one; inside a block the larger
	// im-parity set first (the im-even one on a tie)
	std::vector<int> chmap;
	for (int par = 0; par < 2; ++par) {
		h->off[par] = (int)chmap.size();
		int cnt[2] = {0, 0};
		for (int ch = 0; ch < nch; ++ch) if ((ch % d.n_l) % 2 == par) ++cnt[(ch / d.n_l) & 1];
		h->apar[par] = cnt[1] > cnt[0] ? 1 : 0;
		for (int set = 0; set < 2; ++set) {
			const int ip = set ? 1 - h->apar[par] : h->apar[par];
			for (int ch = 0; ch < nch; ++ch)
				if ((ch % d.n_l) % 2 == par && ((ch / d.n_l) & 1) == ip) chmap.push_back(ch);
		}
		h->nb[par] = (int)chmap.size() - h->off[par];
		h->na[par] = cnt[h->apar[par]];
	}
	int rc;
	if ((rc = dalloc(&h->S, (size_t)N * NE)) || (rc = dalloc(&h->Ri, (size_t)N * NE)) || (rc = dalloc(&h->D, (size_t)N * NE)) ||
		(rc = dalloc(&h->lam[0], nch)) || (rc = dalloc(&h->lam[1], nch)) || (rc = dalloc(&h->lam[2], nch)) || (rc = dalloc(&h->lam[3], nch)) ||
		(rc = dalloc(&h->chmap, (size_t)nch)) ||
		(rc = dalloc(&h->Lrow, (size_t)h->nlh * N * P)) || (rc = dalloc(&h->Dinv, (size_t)h->nlh * N)) ||
		(rc = dalloc(&h->X, nst)) || (rc = dalloc(&h->W, nst)) || (rc = dalloc(&h->U, nst * (NE + 1))) || (rc = dalloc(&h->ntt, (size_t)h->B)) ||
		(rc = dalloc(&h->perm, (size_t)h->B)) || (rc = dalloc(&h->nrm, (size_t)h->B)))
		return fail(rc);
	if (cudaMemcpy(h->chmap, chmap.data(), sizeof(int) * nch, cudaMemcpyHostToDevice) != cudaSuccess) { set_error("upload"); return fail(QPC_ERR_CUDA); }
	// the transforms' GEMMs: exact bf16 digit slices on the tensor cores (default), or the FP64
	// DFMA kernel (QPC_VG_GEMM=dfma)
	if (const char* e = std::getenv("QPC_VG_GEMM")) h->slices = std::strcmp(e, "dfma") != 0;
	if (h->slices) {
		const long J = 2L * N * h->B;
		const long nmax = std::max({(long)h->na[0], (long)h->na[1], (long)(h->nb[0] - h->na[0]), (long)(h->nb[1] - h->na[1]), 1L});
		if ((rc = dalloc(&h->sdB, oz_digits_elems(J, nmax))) || (rc = dalloc(&h->seB, (size_t)J))) return fail(rc);
	}
	// angular eigensystems and the transform matrices, block by block on the device
	std::vector<double> lam[4];
	if ((rc = device_transforms(h, chmap, lam))) return fail(rc);
	if (cudaMemcpy(h->S, S, sizeof(double) * N * NE, cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemcpy(h->Ri, Rinv, sizeof(double) * N * NE, cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemcpy(h->D, D, sizeof(double) * N * NE, cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemcpy(h->Lrow, lrow.data(), sizeof(double) * lrow.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemcpy(h->Dinv, dinv.data(), sizeof(double) * dinv.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemset(h->X, 0, sizeof(double2) * nst) != cudaSuccess) {
		set_error("device upload failed");
		return fail(QPC_ERR_CUDA);
	}
	for (int c = 0; c < 4; ++c)
		if (cudaMemcpy(h->lam[c], lam[c].data(), sizeof(double) * nch, cudaMemcpyHostToDevice) != cudaSuccess) { set_error("upload"); return fail(QPC_ERR_CUDA); }
	*out = h;
	return QPC_OK;
}

int qpc_vgwr_destroy(qpc_vgwr* h)
{
	vg_free(h);
	return QPC_OK;
}

static int vg_copy(qpc_vgwr* h, const double* src, double* dst, cudaMemcpyKind kind)
{
	if (!h || (!src && !dst)) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	cudaSetDevice(h->dev);
	const long total = (long)h->B * h->nch * h->N;
	const size_t bytes = sizeof(double2) * (size_t)total;
	const unsigned nb = (unsigned)((total + 255) / 256);
	// host buffers are copied with the stream idle (bounded wait first): such a copy then
	// never waits for queued work, and a wait that runs out leaves no copy pending
	if (src) {
		if (kind == cudaMemcpyHostToDevice) if (int rc = wait_on(h->st)) return rc;
		QPC_CUDA(cudaMemcpyAsync(h->W, src, bytes, kind, h->st));
		k_vg_permute<<<nb, 256, 0, h->st>>>(h->W, h->X, h->chmap, h->N, h->nch, total, true);
	} else {
		k_vg_permute<<<nb, 256, 0, h->st>>>(h->X, h->W, h->chmap, h->N, h->nch, total, false);
		QPC_CUDA(cudaGetLastError());
		if (kind == cudaMemcpyDeviceToHost) return copy_to_host(dst, h->W, bytes, h->st);
		QPC_CUDA(cudaMemcpyAsync(dst, h->W, bytes, kind, h->st));
	}
	QPC_CUDA(cudaGetLastError());
	return wait_on(h->st);
}

int qpc_vgwr_put(qpc_vgwr* h, const double* coef) { return vg_copy(h, coef, nullptr, cudaMemcpyHostToDevice); }
int qpc_vgwr_get(qpc_vgwr* h, double* coef) { return vg_copy(h, nullptr, coef, cudaMemcpyDeviceToHost); }
int qpc_vgwr_put_device(qpc_vgwr* h, const double* c) { return vg_copy(h, c, nullptr, cudaMemcpyDeviceToDevice); }
int qpc_vgwr_get_device(qpc_vgwr* h, double* c) { return vg_copy(h, nullptr, c, cudaMemcpyDeviceToDevice); }
int qpc_vgwr_dims(qpc_vgwr* h, qpc_dims* dims)
{
	if (!h || !dims) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	*dims = h->d;
	return QPC_OK;
}

// the channel pairs of the dipole observation in the engine's channel order, once per handle
static int dipole_setup(qpc_vgwr* h)
{
	if (h->dpairs) return QPC_OK;
	const int nl = h->d.n_l, nm = h->d.n_m, m0 = h->d.m0;
	std::vector<int> chmap(h->nch), inv(h->nch);
	QPC_CUDA(cudaMemcpy(chmap.data(), h->chmap, sizeof(int) * h->nch, cudaMemcpyDeviceToHost));
	for (int t = 0; t < h->nch; ++t) inv[chmap[t]] = t;
	std::vector<int2> pairs;
	std::vector<double> coef;
	for (int im = 0; im + 1 < nm; ++im)
		for (int il = 0; il < nl; ++il) {
			const long m = m0 + im, l = il + std::labs(m), m2 = m + 1;
			for (int sgn = 1; sgn >= -1; sgn -= 2) {
				const long l2 = l + sgn, il2 = l2 - std::labs(m2);
				if (l2 < 0 || il2 < 0 || il2 >= nl) continue;
				// integrate_sinexp1 (l + 1) and integrate_sinexp2 (l - 1), spherical/utilities/basisfunc.hpp:243-259
				const double c = sgn > 0 ? -std::sqrt(double((l + m + 2) * (l + m + 1)) / double((2 * l + 1) * (2 * l + 3)))
					: std::sqrt(double((l - m) * (l - m - 1)) / double((2 * l + 1) * (2 * l - 1)));
				pairs.push_back(make_int2(inv[im * nl + il], inv[(im + 1) * nl + (int)il2]));
				coef.push_back(c);
			}
		}
	h->ndpairs = (int)pairs.size();
	if (int rc = dalloc(&h->dpairs, std::max<size_t>(pairs.size(), 1))) return rc;
	if (int rc = dalloc(&h->dcoef, std::max<size_t>(coef.size(), 1))) return rc;
	if (int rc = dalloc(&h->dF, (size_t)h->N * (h->P + 1))) return rc;
	h->dnblk = std::max(1, std::min(64, (304 + h->B - 1) / h->B));
	if (int rc = dalloc(&h->dpart, (size_t)h->B * h->dnblk)) return rc;
	if (!pairs.empty()) {
		QPC_CUDA(cudaMemcpy(h->dpairs, pairs.data(), sizeof(int2) * pairs.size(), cudaMemcpyHostToDevice));
		QPC_CUDA(cudaMemcpy(h->dcoef, coef.data(), sizeof(double) * coef.size(), cudaMemcpyHostToDevice));
	}
	return QPC_OK;
}

static int run_impl(qpc_vgwr* h, const double* atab, int64_t ld, const int64_t* nt_field, const int64_t* nt_total,
	const double* F, double* xlist, double* ylist, int64_t ldz)
{
	if (!h || !nt_field || !nt_total) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	cudaSetDevice(h->dev);
	if (int rc = wait_on(h->st)) return rc;
	const int B = h->B;
	long smax = 0;
	bool anyfield = false;
	for (int k = 0; k < B; ++k) {
		if (nt_field[k] < 0 || nt_total[k] < nt_field[k]) { set_error("instance %d: nt_field=%lld nt_total=%lld", k, (long long)nt_field[k], (long long)nt_total[k]); return QPC_ERR_ARGS; }
		if (nt_field[k] > 0) { anyfield = true; if (ld < nt_field[k] + 1) { set_error("ld=%lld < nt_field+1", (long long)ld); return QPC_ERR_ARGS; } }
		smax = std::max<long>(smax, nt_total[k]);
	}
	if (anyfield && !atab) { set_error("atab is NULL"); return QPC_ERR_ARGS; }
	if (F && (!xlist || !ylist || ldz < smax)) { set_error("xlist/ylist NULL or ldz=%lld < max nt_total=%ld", (long long)ldz, smax); return QPC_ERR_ARGS; }
	if (smax == 0) return QPC_OK;
	if (F) {
		if (int rc = dipole_setup(h)) return rc;
		if ((size_t)B * ldz > h->dcap) {
			if (h->dxs) cudaFree(h->dxs);
			if (h->dys) cudaFree(h->dys);
			h->dxs = h->dys = nullptr; h->dcap = 0;
			if (int rc = dalloc(&h->dxs, (size_t)B * ldz)) return rc;
			if (int rc = dalloc(&h->dys, (size_t)B * ldz)) return rc;
			h->dcap = (size_t)B * ldz;
		}
		QPC_CUDA(cudaMemcpyAsync(h->dF, F, sizeof(double) * h->N * (h->P + 1), cudaMemcpyHostToDevice, h->st));
		QPC_CUDA(cudaMemsetAsync(h->dxs, 0, sizeof(double) * B * ldz, h->st));
		QPC_CUDA(cudaMemsetAsync(h->dys, 0, sizeof(double) * B * ldz, h->st));
	}
	const long cap = anyfield ? (long)B * ld * 2 : 2;
	if (cap > h->atab_cap) {
		if (h->atab) cudaFree(h->atab);
		h->atab = nullptr; h->atab_cap = 0;
		if (int rc = dalloc(&h->atab, cap)) return rc;
		h->atab_cap = cap;
	}
	if (anyfield) {
		for (int k = 0; k < B; ++k)
			for (long i = 0; i <= nt_field[k] && nt_field[k] > 0; ++i)
				if (!std::isfinite(atab[((size_t)k * ld + i) * 2]) || !std::isfinite(atab[((size_t)k * ld + i) * 2 + 1])) {
					set_error("non-finite vector potential, instance %d step %ld", k, i);
					return QPC_ERR_ARGS;
				}
		QPC_CUDA(cudaMemcpyAsync(h->atab, atab, sizeof(double) * cap, cudaMemcpyHostToDevice, h->st));
	}
	// instances in decreasing nt_field: the ones in their pulse at step s are a prefix
	std::vector<int> perm(B);
	std::iota(perm.begin(), perm.end(), 0);
	std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) { return nt_field[x] > nt_field[y]; });
	bool ident = true;
	for (int k = 0; k < B; ++k) ident &= perm[k] == k;
	std::vector<long long> ntt(nt_total, nt_total + B);
	QPC_CUDA(cudaMemcpyAsync(h->ntt, ntt.data(), sizeof(long long) * B, cudaMemcpyHostToDevice, h->st));
	QPC_CUDA(cudaMemcpyAsync(h->perm, perm.data(), sizeof(int) * B, cudaMemcpyHostToDevice, h->st));
	if (!ident) if (int rc = permute(h, perm, false)) return rc;
	// instances running (nt_total) at step s: those with nt_total > s; the field-free kernel
	// checks nt_total per instance, and covers the prefix up to the last running one
	h->launches = 0;
	QPC_CUDA(cudaEventRecord(h->ev0, h->st));
	for (long s = 0; s < smax; ++s) {
		int nlive = 0, nff = 0;
		for (int k = 0; k < B; ++k) {
			if (s < nt_field[perm[k]]) nlive = k + 1;
			if (s < nt_total[perm[k]]) nff = k + 1;
		}
		if (F && nff > 0 && h->ndpairs > 0) {
			// the observation before step s (binsrc/sphTDSE.cpp:933-934)
			k_vg_dip_part<<<dim3((unsigned)h->dnblk, (unsigned)nff), DIP_THREADS, 0, h->st>>>(h->X, h->dF, h->dpairs, h->dcoef,
				h->ndpairs, h->N, h->P, h->nch, h->ntt, h->perm, s, h->dpart);
			k_vg_dip_final<<<(unsigned)((nff + 127) / 128), 128, 0, h->st>>>(h->dpart, h->dnblk, nff, h->ntt, h->perm, s, ldz, h->dxs, h->dys);
			h->launches += 2;
		}
		if (int rc = step_dispatch(h, s, anyfield ? ld : 0, nlive, nff)) return rc;
	}
	QPC_CUDA(cudaGetLastError());
	QPC_CUDA(cudaEventRecord(h->ev1, h->st));
	if (!ident) if (int rc = permute(h, perm, true)) return rc;
	if (int rc = wait_on(h->st)) return rc;
	if (h->slices) if (int rc = oz_check(h->st)) return rc;
	cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1);
	prof_collect(h);
	if (F) {
		std::vector<double> xh((size_t)B * ldz), yh((size_t)B * ldz);
		if (int rc = copy_to_host(xh.data(), h->dxs, sizeof(double) * xh.size(), h->st)) return rc;
		if (int rc = copy_to_host(yh.data(), h->dys, sizeof(double) * yh.size(), h->st)) return rc;
		for (int k = 0; k < B; ++k) {
			std::memcpy(xlist + (size_t)perm[k] * ldz, xh.data() + (size_t)k * ldz, sizeof(double) * ldz);
			std::memcpy(ylist + (size_t)perm[k] * ldz, yh.data() + (size_t)k * ldz, sizeof(double) * ldz);
		}
	}
	return QPC_OK;
}

int qpc_vgwr_run(qpc_vgwr* h, const double* atab, int64_t ld, const int64_t* nt_field, const int64_t* nt_total)
{
	return run_impl(h, atab, ld, nt_field, nt_total, nullptr, nullptr, nullptr, 0);
}

int qpc_vgwr_run_dipole(qpc_vgwr* h, const double* atab, int64_t ld, const int64_t* nt_field, const int64_t* nt_total,
	const double* F, double* xlist, double* ylist, int64_t ldz)
{
	if (!F) { set_error("F is NULL"); return QPC_ERR_ARGS; }
	return run_impl(h, atab, ld, nt_field, nt_total, F, xlist, ylist, ldz);
}

int qpc_vgwr_propagate(qpc_vgwr* h, const double* ax_ti, const double* ax_tf, const double* ay_ti, const double* ay_tf)
{
	if (!h || !ax_ti || !ax_tf || !ay_ti || !ay_tf) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	std::vector<double> tab((size_t)h->B * 4);
	for (int k = 0; k < h->B; ++k) {
		tab[(size_t)k * 4 + 0] = ax_ti[k]; tab[(size_t)k * 4 + 1] = ay_ti[k];
		tab[(size_t)k * 4 + 2] = ax_tf[k]; tab[(size_t)k * 4 + 3] = ay_tf[k];
	}
	std::vector<int64_t> one(h->B, 1);
	return qpc_vgwr_run(h, tab.data(), 2, one.data(), one.data());
}

int qpc_vgwr_propagate_free(qpc_vgwr* h)
{
	if (!h) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	std::vector<int64_t> zero(h->B, 0), one(h->B, 1);
	return qpc_vgwr_run(h, nullptr, 1, zero.data(), one.data());
}

int qpc_vgwr_norm(qpc_vgwr* h, double* norm)
{
	if (!h || !norm) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	cudaSetDevice(h->dev);
	k_vg_snorm<<<h->B, 256, 0, h->st>>>(h->X, h->S, h->N, h->P, h->nch, h->nrm);
	QPC_CUDA(cudaGetLastError());
	return copy_to_host(norm, h->nrm, sizeof(double) * h->B, h->st);
}

int qpc_vgwr_set_profiling(qpc_vgwr* h, int on)
{
	if (!h) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	h->profiling = on != 0;
	for (int k = 0; k < 3; ++k) { h->kms[k] = 0.0; h->kcnt[k] = 0; }
	return QPC_OK;
}

int qpc_vgwr_kernel_times(qpc_vgwr* h, double* ms, int64_t* launches)
{
	if (!h || !ms || !launches) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	for (int k = 0; k < 3; ++k) { ms[k] = h->kms[k]; launches[k] = h->kcnt[k]; }
	return QPC_OK;
}

int qpc_vgwr_last_run(qpc_vgwr* h, float* ms, int64_t* launches)
{
	if (!h || !ms || !launches) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	*ms = h->last_ms;
	*launches = h->launches;
	return QPC_OK;
}

} // extern "C"
