// GB300 (sm_103a) engine for the QPC-TDSE Arnoldi (Lanczos) propagator in the
// length gauge: propagator_arnoldi::propagate1 driven by propagator_hc_lgwz
// (spherical/propagator/la_1e.hpp:312-335, 390-444).  One step maps
// w -> exp(-i dt S^-1 H) w in a Krylov space of at most kmax vectors built in
// the S metric, H = H_l (x) 1 + ez R (x) Y10.
//
// A batch holds B wavefunctions on one radial grid; each may carry its own
// Hamiltonian (its own potential) and its own field table and step count.
// Per step and per instance the kernels are
//   k_ar_snorm   |w|_S (and, inside the loop, |v|_S with the breakdown test)
//   k_ar_expand  u_k = v_k / |v_k|_S, v_{k+1} = H u_k, x_i = <u_i|v_{k+1}>
//   k_ar_sinv    v = S^-1 v, forward and backward banded Cholesky sweeps
//   k_ar_orth    v -= x_i u_i (i = k always, others when |x_i|^2 > 4e-27)
//   k_ar_small   exp(-i dt T) e1 b0 for the m x m tridiagonal T (implicit QL)
//   k_ar_combine w = sum_i x_i u_i
// in the reference's order of operations (la_1e.hpp:132-240).  Reductions are
// deterministic: each block writes a partial, and the last block of the
// instance to finish adds the partials in a fixed order.
//
// The state is kept r-major inside the engine, [inst][r][ch] with ch = im n_l + il,
// so that one warp reads 32 consecutive doubles: consecutive channels at one r
// for the band products, and the real and imaginary parts of consecutive
// channels for the S^-1 recurrences (one real recurrence per lane).
// All arithmetic is complex FP64.
#include "qpc_internal.h"
#include "qpc_cuda_util.cuh"
#include <cuda_runtime.h>
#include <cmath>
#include <vector>
#include <algorithm>
#include <cstdlib>

namespace qpc {
namespace {

constexpr int AR_THREADS = 256;
constexpr int AR_PER_THREAD = 4;
constexpr int AR_TILE = AR_THREADS * AR_PER_THREAD; // elements per block of the element-wise kernels
constexpr int AR_KMAX = 32;                          // largest Krylov dimension accepted
constexpr int CH_THREADS = 32;                       // real recurrences per block of k_ar_sinv

// per-instance state of the expansion within one step
enum : int { AR_LIVE = 0, AR_BROKEN = 1, AR_IDLE = 2 };
// device status bits (never a trap)
enum : int { ARS_NONFINITE = 2, ARS_NOCONV = 4, ARS_ZERO = 8 };

struct ar_args {
	int N, P, L, M, m0, nch, nlh, B, kmax, nbe;
	int b0;       // first instance of the group a launch covers (blockIdx.y / blockIdx.x offset)
	long n;       // complex elements per instance
	long hstride; // doubles between the Hamiltonians of consecutive instances (0: shared)
	double dt, emin, emax;
	const double *S, *R, *Lrow, *Lcol, *dinv, *H, *y10;
	double2 *X, *U, *V0, *V1;
	double2* partX;
	double* partN;
	unsigned* cnt;
	double2* xfin;
	double *a, *b, *sfac, *nu0;
	int *msub, *flag;
	double2* xc;
	const double* ez;
	long ld;
	const long long* nt;
	int8_t *crit, *msub_out;
	int* status;
};

__device__ __forceinline__ double2 cmul(double2 x, double2 y)
{
	return make_double2(fma(y.x, x.x, -(y.y * x.y)), fma(y.x, x.y, y.y * x.x));
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 rmul(double2 x, double s) { return make_double2(x.x * s, x.y * s); }
// conj(u) v
__device__ __forceinline__ double2 cdot(double2 u, double2 v)
{
	return make_double2(fma(u.x, v.x, u.y * v.y), fma(u.x, v.y, -(u.y * v.x)));
}

// deterministic block sum (fixed shuffle tree, then warp 0 over the warp sums); valid in thread 0
__device__ double2 block_sum(double2 v, double2* sm)
{
	for (int o = 16; o; o >>= 1) {
		v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
		v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
	}
	const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
	__syncthreads();
	if (l == 0) sm[w] = v;
	__syncthreads();
	double2 r = make_double2(0.0, 0.0);
	if (w == 0) {
		r = l < nw ? sm[l] : make_double2(0.0, 0.0);
		for (int o = 16; o; o >>= 1) {
			r.x += __shfl_xor_sync(0xffffffffu, r.x, o);
			r.y += __shfl_xor_sync(0xffffffffu, r.y, o);
		}
	}
	return r;
}

// after thread 0 wrote this block's partial: true in every thread of the block that
// arrives last among the instance's nb blocks (threadFenceReduction pattern)
__device__ bool arrive_last(unsigned* cnt, int nb)
{
	__shared__ bool last;
	if (threadIdx.x == 0) {
		__threadfence();
		unsigned t = atomicAdd(cnt, 1u);
		last = (t == (unsigned)nb - 1u);
	}
	__syncthreads();
	return last;
}

// fixed-order sum of nb partials by warp 0 (lanes stride, then the shuffle tree); valid in lane 0
__device__ double2 sum_partials(const double2* p, long stride, int nb)
{
	double2 s = make_double2(0.0, 0.0);
	for (int j = threadIdx.x; j < nb; j += 32) s = cadd(s, __ldcg(p + (long)j * stride));
	for (int o = 16; o; o >>= 1) {
		s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
		s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
	}
	return s;
}

// ---------------------------------------------------------------- layout
__global__ void k_ar_to_rmajor(const double2* __restrict__ src, double2* __restrict__ dst, int N, int nch, long total)
{
	long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= total) return;
	long n = (long)N * nch, b = i / n, e = i - b * n;
	int r = (int)(e / nch), ch = (int)(e - (long)r * nch);
	dst[i] = src[b * n + (long)ch * N + r];
}
__global__ void k_ar_to_lmajor(const double2* __restrict__ src, double2* __restrict__ dst, int N, int nch, long total)
{
	long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= total) return;
	long n = (long)N * nch, b = i / n, e = i - b * n;
	int ch = (int)(e / N), r = (int)(e - (long)ch * N);
	dst[i] = src[b * n + (long)r * nch + ch];
}

// ---------------------------------------------------------------- S-norm and breakdown test
// Re sum_e conj(x_e) (S x)_e per instance (operator_rsym::observe, operators/1e.hpp:69-79).
// k < 0: start of a step (construct_sub, la_1e.hpp:132-151): sfac = 1/|w|_S, b[0] = |w|_S,
//        or the instance idles this step (step >= nt).
// k >= 0: end of iteration k (orthogonalize_ip, la_1e.hpp:221-238): nu < 1e-13 ends the
//        expansion with m = k+1; else sfac = 1/sqrt(nu), b[k+1] = sqrt(nu).
__global__ void __launch_bounds__(AR_THREADS) k_ar_snorm(ar_args g, const double2* __restrict__ src, int k, long step)
{
	const int b = g.b0 + blockIdx.y;
	if (k < 0) {
		if (step >= g.nt[b]) {
			if (blockIdx.x == 0 && threadIdx.x == 0) g.flag[b] = AR_IDLE;
			return;
		}
	} else if (g.flag[b] != AR_LIVE) return;
	__shared__ double2 sm[32];
	const int P = g.P, nch = g.nch, N = g.N;
	const double2* x = src + (long)b * g.n;
	double acc = 0.0;
	for (int j = 0; j < AR_PER_THREAD; ++j) {
		long e = (long)blockIdx.x * AR_TILE + j * AR_THREADS + threadIdx.x;
		if (e >= g.n) break;
		int r = (int)(e / nch);
		double2 t = make_double2(0.0, 0.0);
		for (int q = 1; q <= P && q <= r; ++q) {
			double s = g.S[(long)(r - q) * (P + 1) + q];
			double2 v = x[e - (long)q * nch];
			t.x = fma(s, v.x, t.x); t.y = fma(s, v.y, t.y);
		}
		for (int q = 0; q <= P && r + q < N; ++q) {
			double s = g.S[(long)r * (P + 1) + q];
			double2 v = x[e + (long)q * nch];
			t.x = fma(s, v.x, t.x); t.y = fma(s, v.y, t.y);
		}
		double2 c = x[e];
		acc = fma(c.x, t.x, fma(c.y, t.y, acc));
	}
	double2 tot = block_sum(make_double2(acc, 0.0), sm);
	if (threadIdx.x == 0) g.partN[(long)b * g.nbe + blockIdx.x] = tot.x;
	if (!arrive_last(g.cnt + b, g.nbe)) return;
	if (threadIdx.x < 32) {
		double s = 0.0;
		for (int j = threadIdx.x; j < g.nbe; j += 32) s += __ldcg(g.partN + (long)b * g.nbe + j);
		for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
		if (threadIdx.x == 0) {
			g.cnt[b] = 0u;
			const long bb = (long)b * (g.kmax + 1);
			if (k < 0) {
				g.nu0[b] = s;
				if (!(s > 0.0) || !isfinite(s)) {
					atomicOr(g.status, ARS_ZERO);
					g.flag[b] = AR_IDLE;
				} else {
					double nrm = sqrt(s);
					g.sfac[b] = 1.0 / nrm;
					g.b[bb] = nrm;
					g.flag[b] = AR_LIVE;
					g.msub[b] = g.kmax;
				}
			} else if (s < 1e-13) {
				g.b[bb + k + 1] = 0.0;
				g.flag[b] = AR_BROKEN;
				g.msub[b] = k + 1;
			} else {
				double nrm = sqrt(s);
				g.sfac[b] = 1.0 / nrm;
				g.b[bb + k + 1] = nrm;
			}
		}
	}
}

// ---------------------------------------------------------------- expansion
// u_k = sfac * src (stored as U[k]); dst = H u_k (multiply, la_1e.hpp:420-434:
// symb_mul_vecd of H_l, then + (R u_{l-1}) ez y10(m,l-1), + (R u_{l+1}) ez y10(m,l));
// x_i = <u_i|dst> for i <= k (orthogonalize_ip, la_1e.hpp:204-209), a[k] = Re x_k.
// The band sums run on the unscaled src and are scaled once, H (s x) = s (H x): the
// same value to rounding, for a third of the FP64 instructions.
__global__ void __launch_bounds__(AR_THREADS) k_ar_expand(ar_args g, const double2* __restrict__ src, double2* __restrict__ dst,
	int k, long step)
{
	const int b = g.b0 + blockIdx.y;
	if (g.flag[b] != AR_LIVE) return;
	__shared__ double2 sm[32];
	const int P = g.P, nch = g.nch, N = g.N, L = g.L;
	const long n = g.n;
	const double s = g.sfac[b];
	const double ez = g.ez[(long)b * g.ld + step];
	const double2* __restrict__ x = src + (long)b * n;
	double2* y = dst + (long)b * n;
	double2* Uk = g.U + ((long)b * g.kmax + k) * n;
	const double* __restrict__ H = g.H + (long)b * g.hstride;
	const double* __restrict__ Rb = g.R;
	double2 yv[AR_PER_THREAD], uv[AR_PER_THREAD];
#pragma unroll
	for (int j = 0; j < AR_PER_THREAD; ++j) {
		yv[j] = uv[j] = make_double2(0.0, 0.0);
		long e = (long)blockIdx.x * AR_TILE + j * AR_THREADS + threadIdx.x;
		if (e >= n) continue;
		int r = (int)(e / nch), ch = (int)(e - (long)r * nch);
		int im = ch / L, il = ch - im * L;
		int l = il + abs(g.m0 + im);
		double2 ue = rmul(x[e], s);
		Uk[e] = ue;
		uv[j] = ue;
		// H_l band: lower neighbours q ascending, then the row itself and the upper ones
		double2 t = make_double2(0.0, 0.0);
		for (int q = 1; q <= P && q <= r; ++q) {
			double h = H[((long)(r - q) * (P + 1) + q) * g.nlh + l];
			double2 v = x[e - (long)q * nch];
			t.x = fma(v.x, h, t.x); t.y = fma(v.y, h, t.y);
		}
		for (int q = 0; q <= P && r + q < N; ++q) {
			double h = H[((long)r * (P + 1) + q) * g.nlh + l];
			double2 v = x[e + (long)q * nch];
			t.x = fma(v.x, h, t.x); t.y = fma(v.y, h, t.y);
		}
		// R band on the l-1 and l+1 channels of the same m
		double2 t2 = make_double2(0.0, 0.0), t3 = make_double2(0.0, 0.0);
		const bool lo = il > 0, hi = il < L - 1;
		for (int q = 1; q <= P && q <= r; ++q) {
			double rq = Rb[(long)(r - q) * (P + 1) + q];
			long o = e - (long)q * nch;
			if (lo) { double2 v = x[o - 1]; t2.x = fma(v.x, rq, t2.x); t2.y = fma(v.y, rq, t2.y); }
			if (hi) { double2 v = x[o + 1]; t3.x = fma(v.x, rq, t3.x); t3.y = fma(v.y, rq, t3.y); }
		}
		for (int q = 0; q <= P && r + q < N; ++q) {
			double rq = Rb[(long)r * (P + 1) + q];
			long o = e + (long)q * nch;
			if (lo) { double2 v = x[o - 1]; t2.x = fma(v.x, rq, t2.x); t2.y = fma(v.y, rq, t2.y); }
			if (hi) { double2 v = x[o + 1]; t3.x = fma(v.x, rq, t3.x); t3.y = fma(v.y, rq, t3.y); }
		}
		const double clo = lo ? ez * g.y10[im * L + il - 1] : 0.0;
		const double chi = hi ? ez * g.y10[im * L + il] : 0.0;
		double2 acc;
		acc.x = fma(t3.x, chi, fma(t2.x, clo, t.x)) * s;
		acc.y = fma(t3.y, chi, fma(t2.y, clo, t.y)) * s;
		y[e] = acc;
		yv[j] = acc;
	}
	// projections x_i = <u_i|v>, i <= k, one fixed-order block sum each
	double2* part = g.partX + ((long)b * g.nbe + blockIdx.x) * g.kmax;
	for (int i = 0; i <= k; ++i) {
		const double2* Ui = g.U + ((long)b * g.kmax + i) * n;
		double2 acc = make_double2(0.0, 0.0);
		for (int j = 0; j < AR_PER_THREAD; ++j) {
			long e = (long)blockIdx.x * AR_TILE + j * AR_THREADS + threadIdx.x;
			if (e >= n) break;
			double2 ui = (i == k) ? uv[j] : Ui[e];
			acc = cadd(acc, cdot(ui, yv[j]));
		}
		double2 tot = block_sum(acc, sm);
		if (threadIdx.x == 0) part[i] = tot;
	}
	if (!arrive_last(g.cnt + b, g.nbe)) return;
	if (threadIdx.x < 32) {
		for (int i = 0; i <= k; ++i) {
			double2 xi = sum_partials(g.partX + (long)b * g.nbe * g.kmax + i, g.kmax, g.nbe);
			if (threadIdx.x == 0) g.xfin[(long)b * g.kmax + i] = xi;
			if (threadIdx.x == 0 && i == k) g.a[(long)b * g.kmax + k] = xi.x;
		}
		if (threadIdx.x == 0) g.cnt[b] = 0u;
	}
}

// ---------------------------------------------------------------- S^-1
// v = (L L^T)^-1 v per (m,l) channel: ltrb_inv_vecd then utrb_inv_vecd
// (utilities/blas2.hpp:421-433, 1006-1040), the per-channel solve of
// operator_sc::inverse_sub (operators/1e.hpp:1247-1251).  One lane per real
// recurrence (channel, real or imaginary part); the previous P values of each
// sweep stay in registers.  Lrow[r][j-1] = L(r, r-j), Lcol[r][k-1] = L(r+k, r)
// (zero outside the matrix), dinv[r] = 1/L(r,r).  The rows advance in tiles of
// SV_D: the next tile's values are loaded while the current one is solved, and
// the factor rows of the next tile are staged in shared memory by the block.
constexpr int SV_D = 8;

template <int P, bool FWD>
__device__ __forceinline__ void sinv_sweep(const ar_args& g, double* v, long stride, bool act,
	double (*Lt)[SV_D][P + 1])
{
	const int N = g.N;
	const double* __restrict__ Lf = FWD ? g.Lrow : g.Lcol;
	const int ntile = (N + SV_D - 1) / SV_D;
	auto row = [&](int t, int j) { return FWD ? t * SV_D + j : N - 1 - (t * SV_D + j); };
	auto stage = [&](int t, int buf) {
		for (int i = threadIdx.x; i < SV_D * (P + 1); i += blockDim.x) {
			int j = i / (P + 1), c = i - j * (P + 1);
			int r = row(t, j);
			double val = 0.0;
			if (t * SV_D + j < N) val = c < P ? Lf[(long)r * P + c] : g.dinv[r];
			Lt[buf][j][c] = val;
		}
	};
	double w[P];
#pragma unroll
	for (int j = 0; j < P; ++j) w[j] = 0.0;
	double cur[SV_D], nxt[SV_D];
#pragma unroll
	for (int j = 0; j < SV_D; ++j) cur[j] = (act && j < N) ? v[(long)row(0, j) * stride] : 0.0;
	stage(0, 0);
	__syncthreads();
	for (int t = 0; t < ntile; ++t) {
		const int buf = t & 1;
		if (t + 1 < ntile) {
#pragma unroll
			for (int j = 0; j < SV_D; ++j) nxt[j] = (act && (t + 1) * SV_D + j < N) ? v[(long)row(t + 1, j) * stride] : 0.0;
			stage(t + 1, buf ^ 1);
		}
#pragma unroll
		for (int j = 0; j < SV_D; ++j) {
			if (t * SV_D + j < N) {
				double x = cur[j];
#pragma unroll
				for (int q = 0; q < P; ++q) x = fma(-w[q], Lt[buf][j][q], x);
				x *= Lt[buf][j][P];
#pragma unroll
				for (int q = P - 1; q > 0; --q) w[q] = w[q - 1];
				w[0] = x;
				if (act) v[(long)row(t, j) * stride] = x;
			}
		}
		__syncthreads();
#pragma unroll
		for (int j = 0; j < SV_D; ++j) cur[j] = nxt[j];
	}
}

template <int P>
__global__ void __launch_bounds__(CH_THREADS) k_ar_sinv(ar_args g, double2* __restrict__ vbuf)
{
	const int b = g.b0 + blockIdx.y;
	if (g.flag[b] != AR_LIVE) return;
	__shared__ double Lt[2][SV_D][P + 1];
	const int c = blockIdx.x * CH_THREADS + threadIdx.x;
	const bool act = c < 2 * g.nch;
	const long stride = 2L * g.nch;
	double* v = reinterpret_cast<double*>(vbuf + (long)b * g.n) + (act ? c : 0);
	sinv_sweep<P, true>(g, v, stride, act, Lt);
	sinv_sweep<P, false>(g, v, stride, act, Lt);
}

// The same solve with P lanes per real recurrence, column-oriented (for batches too small
// to occupy the GPU one lane per recurrence): lane j of a recurrence holds the pending sum
// of one of the next P rows; when row r is complete its owner's sum is broadcast, every lane
// computes x_r, and each lane adds L(row_j, r) x_r to its own row's sum.  Three FP64
// instructions per row instead of P + 1, on P times as many warps.
template <int P>
__global__ void __launch_bounds__(128) k_ar_sinv_sys(ar_args g, double2* __restrict__ vbuf)
{
	const int b = g.b0 + blockIdx.y;
	if (g.flag[b] != AR_LIVE) return;
	constexpr int CPW = 32 / P;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int cs = lane / P, j = lane - cs * P;
	const int c = (blockIdx.x * (int)(blockDim.x >> 5) + warp) * CPW + cs;
	const bool act = cs < CPW && c < 2 * g.nch;
	const int base = (cs < CPW ? cs : 0) * P;
	const long stride = 2L * g.nch;
	const int N = g.N;
	double* v = reinterpret_cast<double*>(vbuf + (long)b * g.n) + (act ? c : 0);
	const double* __restrict__ Lcol = g.Lcol;
	const double* __restrict__ Lrow = g.Lrow;
	const double* __restrict__ dinv = g.dinv;
	// forward: rows r ascending, owner o = r mod P
	{
		double acc = 0.0, cur[SV_D], nxt[SV_D];
		const int ntile = (N + SV_D - 1) / SV_D;
#pragma unroll
		for (int q = 0; q < SV_D; ++q) cur[q] = (act && q < N) ? v[(long)q * stride] : 0.0;
		int o = 0;
		for (int t = 0; t < ntile; ++t) {
#pragma unroll
			for (int q = 0; q < SV_D; ++q) {
				int r = (t + 1) * SV_D + q;
				nxt[q] = (act && r < N) ? v[(long)r * stride] : 0.0;
			}
#pragma unroll
			for (int q = 0; q < SV_D; ++q) {
				const int r = t * SV_D + q;
				if (r < N) {
					double ao = __shfl_sync(0xffffffffu, acc, base + o);
					double x = (cur[q] - ao) * dinv[r];
					if (j == o) acc = 0.0;
					int k = (j - o - 1 + P) % P + 1;
					acc = fma(Lcol[(long)r * P + k - 1], x, acc);
					if (act && j == o) v[(long)r * stride] = x;
					o = (o + 1 == P) ? 0 : o + 1;
				}
			}
#pragma unroll
			for (int q = 0; q < SV_D; ++q) cur[q] = nxt[q];
		}
	}
	__syncwarp();
	// backward: rows s = N-1-i descending, owner o = i mod P
	{
		double acc = 0.0, cur[SV_D], nxt[SV_D];
		const int ntile = (N + SV_D - 1) / SV_D;
#pragma unroll
		for (int q = 0; q < SV_D; ++q) cur[q] = (act && q < N) ? v[(long)(N - 1 - q) * stride] : 0.0;
		int o = 0;
		for (int t = 0; t < ntile; ++t) {
#pragma unroll
			for (int q = 0; q < SV_D; ++q) {
				int i = (t + 1) * SV_D + q;
				nxt[q] = (act && i < N) ? v[(long)(N - 1 - i) * stride] : 0.0;
			}
#pragma unroll
			for (int q = 0; q < SV_D; ++q) {
				const int i = t * SV_D + q;
				if (i < N) {
					const int sr = N - 1 - i;
					double ao = __shfl_sync(0xffffffffu, acc, base + o);
					double x = (cur[q] - ao) * dinv[sr];
					if (j == o) acc = 0.0;
					int k = (j - o - 1 + P) % P + 1;
					acc = fma(Lrow[(long)sr * P + k - 1], x, acc);
					if (act && j == o) v[(long)sr * stride] = x;
					o = (o + 1 == P) ? 0 : o + 1;
				}
			}
#pragma unroll
			for (int q = 0; q < SV_D; ++q) cur[q] = nxt[q];
		}
	}
}

// ---------------------------------------------------------------- Gram-Schmidt
// v -= u_i x_i for i <= k with i == k or |x_i|^2 > 4e-27, i ascending (la_1e.hpp:212-219)
__global__ void __launch_bounds__(AR_THREADS) k_ar_orth(ar_args g, double2* __restrict__ vbuf, int k)
{
	const int b = g.b0 + blockIdx.y;
	if (g.flag[b] != AR_LIVE) return;
	__shared__ double2 xs[AR_KMAX];
	__shared__ int use[AR_KMAX];
	if (threadIdx.x <= k) {
		double2 xi = g.xfin[(long)b * g.kmax + threadIdx.x];
		xs[threadIdx.x] = xi;
		use[threadIdx.x] = ((int)threadIdx.x == k) || (xi.x * xi.x + xi.y * xi.y > 4e-27);
	}
	__syncthreads();
	const long n = g.n;
	double2* v = vbuf + (long)b * n;
	for (int j = 0; j < AR_PER_THREAD; ++j) {
		long e = (long)blockIdx.x * AR_TILE + j * AR_THREADS + threadIdx.x;
		if (e >= n) break;
		double2 t = v[e];
		for (int i = 0; i <= k; ++i)
			if (use[i]) t = csub(t, cmul(g.U[((long)b * g.kmax + i) * n + e], xs[i]));
		v[e] = t;
	}
}

// ---------------------------------------------------------------- Krylov-space propagation
// propagate_sub (la_1e.hpp:153-174) and criterion (la_1e.hpp:296-310), one warp per
// instance.  The m x m tridiagonal (a[0..m), b[1..m)) is diagonalised by the implicit
// QL iteration with Wilkinson shifts (Bowdler, Martin, Reinsch and Wilkinson, Numer.
// Math. 11 (1968) 293-306).  Every lane runs the same scalar recurrence on its own
// copy of (d, e); lane j applies the rotations to row j of the eigenvector matrix.
// Then x_j = b0 sum_i z_i[0] exp(-i dt d_i) z_i[j].
__global__ void __launch_bounds__(32) k_ar_small(ar_args g, long step)
{
	const int b = g.b0 + blockIdx.x, lane = threadIdx.x;
	const int fl = g.flag[b];
	if (fl == AR_IDLE) return;
	const int m = fl == AR_BROKEN ? g.msub[b] : g.kmax;
	double d[AR_KMAX], e[AR_KMAX], z[AR_KMAX];
	for (int i = 0; i < m; ++i) {
		d[i] = g.a[(long)b * g.kmax + i];
		e[i] = i + 1 < m ? g.b[(long)b * (g.kmax + 1) + i + 1] : 0.0;
		z[i] = (i == lane) ? 1.0 : 0.0;
	}
	bool ok = true;
	for (int l = 0; l < m && ok; ++l) {
		int iter = 0, mm;
		for (;;) {
			for (mm = l; mm < m - 1; ++mm) {
				double dd = fabs(d[mm]) + fabs(d[mm + 1]);
				if (fabs(e[mm]) <= 1e-300 || fabs(e[mm]) + dd == dd) break;
			}
			if (mm == l) break;
			if (iter++ == 60) { ok = false; break; }
			double gg = (d[l + 1] - d[l]) / (2.0 * e[l]);
			double r = hypot(gg, 1.0);
			gg = d[mm] - d[l] + e[l] / (gg + (gg >= 0 ? r : -r));
			double s = 1.0, c = 1.0, pp = 0.0;
			int i;
			bool underflow = false;
			for (i = mm - 1; i >= l; --i) {
				double f = s * e[i], bb = c * e[i];
				r = hypot(f, gg);
				e[i + 1] = r;
				if (r == 0.0) {
					d[i + 1] -= pp;
					e[mm] = 0.0;
					underflow = true;
					break;
				}
				s = f / r;
				c = gg / r;
				gg = d[i + 1] - pp;
				r = (d[i] - gg) * s + 2.0 * c * bb;
				pp = s * r;
				d[i + 1] = gg + pp;
				gg = c * r - bb;
				double zf = z[i + 1];
				z[i + 1] = s * z[i] + c * zf;
				z[i] = c * z[i] - s * zf;
			}
			if (underflow) continue;
			d[l] -= pp;
			e[l] = gg;
			e[mm] = 0.0;
		}
	}
	if (!ok) {
		if (lane == 0) atomicOr(g.status, ARS_NOCONV);
		return;
	}
	// lane j holds z[i] = component j of eigenvector i
	const double b0 = g.b[(long)b * (g.kmax + 1)];
	double2 xj = make_double2(0.0, 0.0);
	for (int i = 0; i < m; ++i) {
		double z0 = __shfl_sync(0xffffffffu, z[i], 0);
		double sn, cs;
		sincos(-(g.dt * d[i]), &sn, &cs);
		double2 wi = make_double2(z0 * cs, z0 * sn);
		xj = i == 0 ? rmul(wi, z[i]) : cadd(xj, rmul(wi, z[i]));
	}
	xj = rmul(xj, b0);
	if (lane < m) g.xc[(long)b * g.kmax + lane] = xj;
	double2 xl = make_double2(__shfl_sync(0xffffffffu, xj.x, m - 1), __shfl_sync(0xffffffffu, xj.y, m - 1));
	if (lane == 0 && step < g.ld) {
		double eps = m > 1 ? xl.x * xl.x + xl.y * xl.y : 0.0;
		if (g.crit) g.crit[(long)b * g.ld + step] = (int8_t)(eps > g.emax ? 0 : eps > g.emin ? 1 : 2);
		if (g.msub_out) g.msub_out[(long)b * g.ld + step] = (int8_t)m;
	}
}

// w = sum_{i<m} u_i x_i (eliminate_sub, la_1e.hpp:176-193)
__global__ void __launch_bounds__(AR_THREADS) k_ar_combine(ar_args g)
{
	const int b = g.b0 + blockIdx.y;
	const int fl = g.flag[b];
	if (fl == AR_IDLE) return;
	const int m = fl == AR_BROKEN ? g.msub[b] : g.kmax;
	__shared__ double2 xs[AR_KMAX];
	if (threadIdx.x < m) xs[threadIdx.x] = g.xc[(long)b * g.kmax + threadIdx.x];
	__syncthreads();
	const long n = g.n;
	bool bad = false;
	for (int j = 0; j < AR_PER_THREAD; ++j) {
		long e = (long)blockIdx.x * AR_TILE + j * AR_THREADS + threadIdx.x;
		if (e >= n) break;
		const double2* U = g.U + (long)b * g.kmax * n + e;
		double2 w = cmul(U[0], xs[0]);
		for (int i = 1; i < m; ++i) w = cadd(w, cmul(U[(long)i * n], xs[i]));
		g.X[(long)b * n + e] = w;
		bad |= !isfinite(w.x) || !isfinite(w.y);
	}
	if (bad) atomicOr(g.status, ARS_NONFINITE);
}

} // namespace

} // namespace qpc

using namespace qpc;

struct qpc_arnoldi {
	int dev = 0;
	qpc_dims d{};
	int P = 0, nch = 0, nlh = 0, kmax = 0, nbe = 0, hper = 0;
	long n = 0;
	double dt = 0, emin = 0, emax = 0;
	cudaStream_t stream = nullptr, stream2 = nullptr;	// stream2: second instance group (n_inst >= 2)
	cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
	double *S = nullptr, *R = nullptr, *Lrow = nullptr, *Lcol = nullptr, *dinv = nullptr, *H = nullptr, *y10 = nullptr;
	double2 *X = nullptr, *U = nullptr, *V0 = nullptr, *V1 = nullptr, *tmp = nullptr;
	double2* partX = nullptr;
	double* partN = nullptr;
	unsigned* cnt = nullptr;
	double2 *xfin = nullptr, *xc = nullptr;
	double *a = nullptr, *b = nullptr, *sfac = nullptr, *nu0 = nullptr;
	int *msub = nullptr, *flag = nullptr, *status = nullptr;
	double* ez = nullptr;
	long ez_cap = 0;
	long long* nt = nullptr;
	int8_t *crit = nullptr, *msub_out = nullptr;
	long crit_cap = 0;
	float last_ms = 0.f;
	long launches = 0;
};

namespace {

void ar_free(qpc_arnoldi* h)
{
	if (!h) return;
	cudaSetDevice(h->dev);
	void* ptrs[] = {h->S, h->R, h->Lrow, h->Lcol, h->dinv, h->H, h->y10, h->X, h->U, h->V0, h->V1, h->tmp, h->partX, h->partN,
		h->cnt, h->xfin, h->xc, h->a, h->b, h->sfac, h->nu0, h->msub, h->flag, h->status, h->ez, h->nt, h->crit, h->msub_out};
	for (void* p : ptrs)
		if (p) cudaFree(p);
	if (h->ev0) cudaEventDestroy(h->ev0);
	if (h->ev1) cudaEventDestroy(h->ev1);
	if (h->ev2) cudaEventDestroy(h->ev2);
	if (h->stream) cudaStreamDestroy(h->stream);
	if (h->stream2) cudaStreamDestroy(h->stream2);
	delete h;
}

ar_args make_args(qpc_arnoldi* h)
{
	ar_args g{};
	g.N = h->d.n_r; g.P = h->P; g.L = h->d.n_l; g.M = h->d.n_m; g.m0 = h->d.m0; g.nch = h->nch; g.nlh = h->nlh;
	g.B = h->d.n_inst; g.kmax = h->kmax; g.nbe = h->nbe; g.n = h->n; g.b0 = 0;
	g.hstride = h->hper ? (long)h->d.n_r * (h->P + 1) * h->nlh : 0;
	g.dt = h->dt; g.emin = h->emin; g.emax = h->emax;
	g.S = h->S; g.R = h->R; g.Lrow = h->Lrow; g.Lcol = h->Lcol; g.dinv = h->dinv; g.H = h->H; g.y10 = h->y10;
	g.X = h->X; g.U = h->U; g.V0 = h->V0; g.V1 = h->V1;
	g.partX = h->partX; g.partN = h->partN; g.cnt = h->cnt; g.xfin = h->xfin;
	g.a = h->a; g.b = h->b; g.sfac = h->sfac; g.nu0 = h->nu0; g.msub = h->msub; g.flag = h->flag; g.xc = h->xc;
	g.ez = h->ez; g.nt = h->nt; g.crit = h->crit; g.msub_out = h->msub_out; g.status = h->status;
	return g;
}

void launch_sinv(const ar_args& g, int Bg, double2* v, cudaStream_t st)
{
	// one lane per recurrence when that fills the GPU, else P lanes per recurrence
	const long chains = 2L * g.nch * Bg;
	const char* e = getenv("QPC_AR_SINV");
	const bool sys = e ? atoi(e) == 2 : chains < 32L * 304;
	if (sys && g.P >= 2) {
		const int cpw = 32 / g.P;
		dim3 gs((unsigned)((2 * g.nch + 4 * cpw - 1) / (4 * cpw)), Bg);
		switch (g.P) {
		case 2: k_ar_sinv_sys<2><<<gs, 128, 0, st>>>(g, v); return;
		case 3: k_ar_sinv_sys<3><<<gs, 128, 0, st>>>(g, v); return;
		case 4: k_ar_sinv_sys<4><<<gs, 128, 0, st>>>(g, v); return;
		case 5: k_ar_sinv_sys<5><<<gs, 128, 0, st>>>(g, v); return;
		case 6: k_ar_sinv_sys<6><<<gs, 128, 0, st>>>(g, v); return;
		case 7: k_ar_sinv_sys<7><<<gs, 128, 0, st>>>(g, v); return;
		default: k_ar_sinv_sys<8><<<gs, 128, 0, st>>>(g, v); return;
		}
	}
	dim3 grid((2 * g.nch + CH_THREADS - 1) / CH_THREADS, Bg);
	switch (g.P) {
	case 1: k_ar_sinv<1><<<grid, CH_THREADS, 0, st>>>(g, v); break;
	case 2: k_ar_sinv<2><<<grid, CH_THREADS, 0, st>>>(g, v); break;
	case 3: k_ar_sinv<3><<<grid, CH_THREADS, 0, st>>>(g, v); break;
	case 4: k_ar_sinv<4><<<grid, CH_THREADS, 0, st>>>(g, v); break;
	case 5: k_ar_sinv<5><<<grid, CH_THREADS, 0, st>>>(g, v); break;
	case 6: k_ar_sinv<6><<<grid, CH_THREADS, 0, st>>>(g, v); break;
	case 7: k_ar_sinv<7><<<grid, CH_THREADS, 0, st>>>(g, v); break;
	default: k_ar_sinv<8><<<grid, CH_THREADS, 0, st>>>(g, v); break;
	}
}

// one Arnoldi step of instances [g.b0, g.b0 + Bg) on stream st: 4 kmax launches
long launch_step(qpc_arnoldi* h, const ar_args& g, int Bg, cudaStream_t st, long step)
{
	dim3 ge(g.nbe, Bg);
	long nl = 0;
	k_ar_snorm<<<ge, AR_THREADS, 0, st>>>(g, h->X, -1, step); ++nl;
	double2* src = h->X;
	for (int k = 0; k < g.kmax; ++k) {
		double2* dst = (k & 1) ? h->V1 : h->V0;
		k_ar_expand<<<ge, AR_THREADS, 0, st>>>(g, src, dst, k, step); ++nl;
		if (k == g.kmax - 1) break; // u_kmax is never used (eliminate_sub sums i < m)
		launch_sinv(g, Bg, dst, st); ++nl;
		k_ar_orth<<<ge, AR_THREADS, 0, st>>>(g, dst, k); ++nl;
		k_ar_snorm<<<ge, AR_THREADS, 0, st>>>(g, dst, k, step); ++nl;
		src = dst;
	}
	k_ar_small<<<Bg, 32, 0, st>>>(g, step); ++nl;
	k_ar_combine<<<ge, AR_THREADS, 0, st>>>(g); ++nl;
	return nl;
}

int read_status(qpc_arnoldi* h)
{
	int st = 0;
	if (int rc = copy_to_host(&st, h->status, sizeof(int), h->stream)) return rc;
	QPC_CUDA(cudaMemsetAsync(h->status, 0, sizeof(int), h->stream));
	if (int rc = wait_on(h->stream)) return rc;
	if (st & ARS_ZERO) { set_error("a wavefunction has zero or non-finite S-norm"); return QPC_ERR_NUMERIC; }
	if (st & ARS_NOCONV) { set_error("Krylov-space eigenproblem did not converge"); return QPC_ERR_NUMERIC; }
	if (st & ARS_NONFINITE) { set_error("non-finite value in the state"); return QPC_ERR_NUMERIC; }
	return QPC_OK;
}

} // namespace

extern "C" {

int qpc_arnoldi_create(const qpc_dims* dims, const double* S, const double* R, const double* H, int32_t h_per_instance,
	const double* y10, double dt, int32_t kmax, double emin, double emax, qpc_arnoldi** out)
{
	if (!out) { set_error("out is NULL"); return QPC_ERR_ARGS; }
	*out = nullptr;
	if (!dims || !S || !R || !H || !y10) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	const qpc_dims d = *dims;
	if (d.p < 1 || d.p > QPC_MAX_RANK || d.n_r < 2 * d.p + 2 || d.n_l < 1 || d.n_m < 1 || d.n_inst < 1 || d.n_inst > 65535) {
		set_error("bad dims n_r=%d p=%d n_l=%d n_m=%d n_inst=%d", d.n_r, d.p, d.n_l, d.n_m, d.n_inst);
		return QPC_ERR_ARGS;
	}
	if (kmax < 1 || kmax > AR_KMAX) { set_error("kmax=%d outside [1, %d]", kmax, AR_KMAX); return QPC_ERR_ARGS; }
	// arnoldi_workspace's constructor check (la_1e.hpp:58-61)
	if (!(emin <= emax) || !(emin > 0) || !(emax > 0)) { set_error("invalid parameters for arnoldi propagator (emin=%g emax=%g)", emin, emax); return QPC_ERR_ARGS; }
	if (!(dt > 0) || !std::isfinite(dt)) { set_error("dt=%g", dt); return QPC_ERR_ARGS; }
	int dev = 0;
	if (int rc = check_device(&dev)) return rc;
	qpc_arnoldi* h = new (std::nothrow) qpc_arnoldi;
	if (!h) { set_error("host allocation"); return QPC_ERR_NOMEM; }
	auto fail = [&](int rc) { ar_free(h); return rc; };
	h->dev = dev;
	h->d = d;
	h->P = d.p;
	h->nch = d.n_m * d.n_l;
	const int mmax = std::max(std::abs(d.m0), std::abs(d.m0 + d.n_m - 1));
	h->nlh = mmax + d.n_l;
	h->kmax = kmax;
	h->n = (long)h->nch * d.n_r;
	h->nbe = (int)((h->n + AR_TILE - 1) / AR_TILE);
	h->hper = h_per_instance ? 1 : 0;
	h->dt = dt; h->emin = emin; h->emax = emax;
	const int N = d.n_r, P = d.p, NE = P + 1, B = d.n_inst;
	// Cholesky factor of S in both sweep orders
	std::vector<double> Lc((size_t)N * NE);
	int bad = qpc_cholesky_band(N, P, S, Lc.data());
	if (bad) { set_error("S is not positive definite (pivot %d)", bad); return fail(QPC_ERR_SINGULAR); }
	std::vector<double> lrow((size_t)N * P, 0.0), lcol((size_t)N * P, 0.0), di(N);
	for (int r = 0; r < N; ++r) {
		di[r] = 1.0 / Lc[(size_t)r * NE];
		for (int j = 1; j <= P; ++j) {
			if (r - j >= 0) lrow[(size_t)r * P + j - 1] = Lc[(size_t)(r - j) * NE + j];
			if (r + j < N) lcol[(size_t)r * P + j - 1] = Lc[(size_t)r * NE + j];
		}
	}
	// Hamiltonian bands r-major: Hr[hs][r][k][l]
	const int nhs = h->hper ? B : 1;
	std::vector<double> Hr((size_t)nhs * N * NE * h->nlh);
	for (int hs = 0; hs < nhs; ++hs)
		for (int l = 0; l < h->nlh; ++l)
			for (int r = 0; r < N; ++r)
				for (int k = 0; k < NE; ++k) {
					double v = H[(((size_t)hs * h->nlh + l) * N + r) * NE + k];
					if (!std::isfinite(v)) { set_error("non-finite H"); return fail(QPC_ERR_ARGS); }
					Hr[(((size_t)hs * N + r) * NE + k) * h->nlh + l] = v;
				}
	int rc = 0;
	if ((cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess) { set_error("cudaStreamCreateWithFlags failed"); return fail(QPC_ERR_CUDA); }
	if ((cudaEventCreate(&h->ev0)) != cudaSuccess) { set_error("cudaEventCreate failed"); return fail(QPC_ERR_CUDA); }
	if ((cudaEventCreate(&h->ev1)) != cudaSuccess) { set_error("cudaEventCreate failed"); return fail(QPC_ERR_CUDA); }
	if ((cudaEventCreateWithFlags(&h->ev2, cudaEventDisableTiming)) != cudaSuccess) { set_error("cudaEventCreateWithFlags failed"); return fail(QPC_ERR_CUDA); }
	if (B >= 2 && !(getenv("QPC_STREAMS") && atoi(getenv("QPC_STREAMS")) == 1))
		if ((cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking)) != cudaSuccess) { set_error("cudaStreamCreateWithFlags failed"); return fail(QPC_ERR_CUDA); }
	const long nst = (long)B * h->n;
	if ((rc = dalloc(&h->S, (size_t)N * NE)) || (rc = dalloc(&h->R, (size_t)N * NE)) || (rc = dalloc(&h->Lrow, (size_t)N * P)) ||
		(rc = dalloc(&h->Lcol, (size_t)N * P)) || (rc = dalloc(&h->dinv, (size_t)N)) || (rc = dalloc(&h->H, Hr.size())) ||
		(rc = dalloc(&h->y10, (size_t)d.n_m * d.n_l)) || (rc = dalloc(&h->X, nst)) || (rc = dalloc(&h->U, nst * kmax)) ||
		(rc = dalloc(&h->V0, nst)) || (rc = dalloc(&h->V1, nst)) || (rc = dalloc(&h->tmp, nst)) ||
		(rc = dalloc(&h->partX, (size_t)B * h->nbe * kmax)) || (rc = dalloc(&h->partN, (size_t)B * h->nbe)) ||
		(rc = dalloc(&h->cnt, (size_t)B)) || (rc = dalloc(&h->xfin, (size_t)B * kmax)) || (rc = dalloc(&h->xc, (size_t)B * kmax)) ||
		(rc = dalloc(&h->a, (size_t)B * kmax)) || (rc = dalloc(&h->b, (size_t)B * (kmax + 1))) || (rc = dalloc(&h->sfac, (size_t)B)) || (rc = dalloc(&h->nu0, (size_t)B)) ||
		(rc = dalloc(&h->msub, (size_t)B)) || (rc = dalloc(&h->flag, (size_t)B)) || (rc = dalloc(&h->status, 1)) ||
		(rc = dalloc(&h->nt, (size_t)B)))
		return fail(rc);
	if (cudaMemcpy(h->S, S, sizeof(double) * N * NE, cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemcpy(h->R, R, sizeof(double) * N * NE, cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemcpy(h->Lrow, lrow.data(), sizeof(double) * lrow.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemcpy(h->Lcol, lcol.data(), sizeof(double) * lcol.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemcpy(h->dinv, di.data(), sizeof(double) * N, cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemcpy(h->H, Hr.data(), sizeof(double) * Hr.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemcpy(h->y10, y10, sizeof(double) * d.n_m * d.n_l, cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemset(h->X, 0, sizeof(double2) * nst) != cudaSuccess || cudaMemset(h->cnt, 0, sizeof(unsigned) * B) != cudaSuccess ||
		cudaMemset(h->status, 0, sizeof(int)) != cudaSuccess) {
		set_error("device upload failed");
		return fail(QPC_ERR_CUDA);
	}
	*out = h;
	return QPC_OK;
}

int qpc_arnoldi_destroy(qpc_arnoldi* h)
{
	ar_free(h);
	return QPC_OK;
}

static int ar_transfer(qpc_arnoldi* h, const double* src, double* dst, bool put, cudaMemcpyKind kind)
{
	cudaSetDevice(h->dev);
	const long nst = (long)h->d.n_inst * h->n;
	const int tb = 256;
	const unsigned nb = (unsigned)((nst + tb - 1) / tb);
	// host buffers are copied with the stream idle (bounded wait first): such a copy then
	// never waits for queued work, and a wait that runs out leaves no copy pending
	if (put) {
		if (kind == cudaMemcpyHostToDevice) if (int rc = wait_on(h->stream)) return rc;
		QPC_CUDA(cudaMemcpyAsync(h->tmp, src, sizeof(double2) * nst, kind, h->stream));
		k_ar_to_rmajor<<<nb, tb, 0, h->stream>>>(h->tmp, h->X, h->d.n_r, h->nch, nst);
	} else {
		k_ar_to_lmajor<<<nb, tb, 0, h->stream>>>(h->X, h->tmp, h->d.n_r, h->nch, nst);
		QPC_CUDA(cudaGetLastError());
		if (kind == cudaMemcpyDeviceToHost) return copy_to_host(dst, h->tmp, sizeof(double2) * nst, h->stream);
		QPC_CUDA(cudaMemcpyAsync(dst, h->tmp, sizeof(double2) * nst, kind, h->stream));
	}
	QPC_CUDA(cudaGetLastError());
	return wait_on(h->stream);
}

int qpc_arnoldi_put(qpc_arnoldi* h, const double* coef)
{
	if (!h || !coef) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	return ar_transfer(h, coef, nullptr, true, cudaMemcpyHostToDevice);
}

int qpc_arnoldi_get(qpc_arnoldi* h, double* coef)
{
	if (!h || !coef) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	return ar_transfer(h, nullptr, coef, false, cudaMemcpyDeviceToHost);
}

int qpc_arnoldi_put_device(qpc_arnoldi* h, const double* dev_coef)
{
	if (!h || !dev_coef) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	return ar_transfer(h, dev_coef, nullptr, true, cudaMemcpyDeviceToDevice);
}

int qpc_arnoldi_get_device(qpc_arnoldi* h, double* dev_coef)
{
	if (!h || !dev_coef) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	return ar_transfer(h, nullptr, dev_coef, false, cudaMemcpyDeviceToDevice);
}

int qpc_arnoldi_run(qpc_arnoldi* h, const double* ez, int64_t ld, const int64_t* nt, int8_t* crit, int8_t* msub)
{
	if (!h || !ez || !nt) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	cudaSetDevice(h->dev);
	const int B = h->d.n_inst;
	long ntmax = 0;
	for (int k = 0; k < B; ++k) {
		if (nt[k] < 0 || nt[k] > ld) { set_error("instance %d: nt=%lld outside [0, ld=%lld]", k, (long long)nt[k], (long long)ld); return QPC_ERR_ARGS; }
		for (long s = 0; s < nt[k]; ++s)
			if (!std::isfinite(ez[(size_t)k * ld + s])) { set_error("non-finite field value, instance %d step %ld", k, s); return QPC_ERR_ARGS; }
		ntmax = std::max<long>(ntmax, nt[k]);
	}
	if (ntmax == 0) return QPC_OK;
	const long cap = (long)B * ld;
	if (cap > h->ez_cap) {
		if (h->ez) cudaFree(h->ez);
		h->ez = nullptr; h->ez_cap = 0;
		if (int rc = dalloc(&h->ez, cap)) return rc;
		h->ez_cap = cap;
	}
	if ((crit || msub) && cap > h->crit_cap) {
		// (re)allocated below; filled with -1 for the steps an instance does not take
		if (h->crit) cudaFree(h->crit);
		if (h->msub_out) cudaFree(h->msub_out);
		h->crit = h->msub_out = nullptr; h->crit_cap = 0;
		if (int rc = dalloc(&h->crit, cap)) return rc;
		if (int rc = dalloc(&h->msub_out, cap)) return rc;
		h->crit_cap = cap;
	}
	std::vector<long long> ntl(nt, nt + B);
	if (int rc = wait_on(h->stream)) return rc;
	QPC_CUDA(cudaMemcpyAsync(h->ez, ez, sizeof(double) * cap, cudaMemcpyHostToDevice, h->stream));
	QPC_CUDA(cudaMemcpyAsync(h->nt, ntl.data(), sizeof(long long) * B, cudaMemcpyHostToDevice, h->stream));
	ar_args g = make_args(h);
	g.ld = ld;
	if (crit || msub) {
		QPC_CUDA(cudaMemsetAsync(h->crit, 0xff, cap, h->stream));
		QPC_CUDA(cudaMemsetAsync(h->msub_out, 0xff, cap, h->stream));
	} else g.crit = g.msub_out = nullptr;
	long nl = 0;
	// two instance groups on two streams: the latency-bound S^-1 sweeps of one group
	// overlap the band products of the other (instances never interact)
	const int ng = h->stream2 ? 2 : 1;
	int gb[3] = {0, ng == 2 ? (B + 1) / 2 : B, B};
	cudaStream_t gs[2] = {h->stream, h->stream2};
	QPC_CUDA(cudaEventRecord(h->ev0, h->stream));
	if (ng == 2) QPC_CUDA(cudaStreamWaitEvent(h->stream2, h->ev0, 0));
	for (long s = 0; s < ntmax; ++s)
		for (int q = 0; q < ng; ++q) {
			ar_args gq = g;
			gq.b0 = gb[q];
			nl += launch_step(h, gq, gb[q + 1] - gb[q], gs[q], s);
		}
	QPC_CUDA(cudaGetLastError());
	if (ng == 2) {
		QPC_CUDA(cudaEventRecord(h->ev2, h->stream2));
		QPC_CUDA(cudaStreamWaitEvent(h->stream, h->ev2, 0));
	}
	QPC_CUDA(cudaEventRecord(h->ev1, h->stream));
	if (int rc = wait_on(h->stream)) return rc;
	cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1);
	h->launches = nl;
	if (crit) if (int rc = copy_to_host(crit, h->crit, cap, h->stream)) return rc;
	if (msub) if (int rc = copy_to_host(msub, h->msub_out, cap, h->stream)) return rc;
	return read_status(h);
}

int qpc_arnoldi_propagate(qpc_arnoldi* h, const double* ez, int8_t* crit)
{
	if (!h || !ez) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	std::vector<int64_t> ones(h->d.n_inst, 1);
	return qpc_arnoldi_run(h, ez, 1, ones.data(), crit, nullptr);
}

int qpc_arnoldi_norm(qpc_arnoldi* h, double* norm)
{
	if (!h || !norm) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	cudaSetDevice(h->dev);
	const int B = h->d.n_inst;
	// one S-norm pass with every instance live at "step 0" of a one-step table
	std::vector<long long> one(B, 1);
	if (int rc = wait_on(h->stream)) return rc;
	QPC_CUDA(cudaMemcpyAsync(h->nt, one.data(), sizeof(long long) * B, cudaMemcpyHostToDevice, h->stream));
	ar_args g = make_args(h);
	k_ar_snorm<<<dim3(h->nbe, B), AR_THREADS, 0, h->stream>>>(g, h->X, -1, 0);
	QPC_CUDA(cudaGetLastError());
	std::vector<double> nu(B);
	if (int rc = copy_to_host(nu.data(), h->nu0, sizeof(double) * B, h->stream)) return rc;
	QPC_CUDA(cudaMemsetAsync(h->status, 0, sizeof(int), h->stream));
	if (int rc = wait_on(h->stream)) return rc;
	for (int k = 0; k < B; ++k) norm[k] = nu[k];
	return QPC_OK;
}

int qpc_arnoldi_last_run(qpc_arnoldi* h, float* ms, int64_t* launches)
{
	if (!h || !ms || !launches) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	*ms = h->last_ms;
	*launches = h->launches;
	return QPC_OK;
}

} // extern "C"
