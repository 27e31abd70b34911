// GB300 (sm_103a) propagation engine for the QPC-TDSE length-gauge
// Crank-Nicolson step, propagator_cn_hc_lgwz (spherical/propagator/cn_1e.hpp:549-619).
//
// One reference step is  U = C(f_tf) F C(f_ti)  with
//   C(f) = P^T M(f) P,  M(f) = (S + i b R)^-1 (S - i b R) per eigen-channel of Y10
//        (b = lambda f dt/4, cn_propagate_kernel_avx1, propagate.hpp:3-98),
//   F    = (S + i dt/2 H_l)^-1 (S - i dt/2 H_l) per (m,l) channel
//        (cn_hc_propagate0, propagate.hpp:311-331).
// The engine computes exactly these operators, restructured for a GPU whose
// FP64 pipe (~1.2 TFLOP/s on GB300, one warp instruction per ~64 cycles per
// SM sub-partition) is the binding resource:
//   * (S + i b R)^-1 (S - i b R) z = 2 (S + i b R)^-1 (S z) - z, and likewise for
//     F: the right-hand side is a real band times a complex vector, half the
//     FP64 work of the complex band the reference multiplies by.
//   * Y10 has zero diagonal, so its eigenvalues pair as +-s with eigenvectors
//     v and D v, D = diag((-1)^il).  Then S - i b R for -s is the complex
//     conjugate of S + i b R for +s: one LDL^T factorisation serves both
//     channels (the second solve runs on conjugated data), and the l-space
//     transform splits into even-l and odd-l halves (E +- O), half the FP64.
//   * Over a run, C(f(t_i)) closes step i-1 and opens step i, and P P^T = I
//     between them: the run applies P, M(f(t_i))^2 and P^T once per step
//     instead of P M P^T twice.  The factorisation depends only on the field
//     table, so it is computed for several steps ahead in one wide launch.
//   * Each complex recurrence is split over two lanes (real part, imaginary
//     part) and the state is kept r-major, [inst][m][r][l], so that the 32
//     lanes of a warp read 32 consecutive doubles.
// All arithmetic is complex FP64.  Results agree with the reference to
// rounding; the tests hold them to 1e-10 relative L2 after full pulses.
#include "qpc_internal.h"
#include "qpc_cuda_util.cuh"
#include <cuda_runtime.h>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <vector>
#include <algorithm>
#include <numeric>
#include <string>
#include <time.h>
#include <thread>
#include <mutex>
#include <atomic>
#include <functional>
#include <map>
#include <cstdlib>
#include "qpc_chain.cuh"
#include "qpc_ltrans.cuh"

namespace qpc {

static thread_local char g_err[512] = "";
void set_error(const char* fmt, ...)
{
	va_list ap; va_start(ap, fmt);
	vsnprintf(g_err, sizeof(g_err), fmt, ap);
	va_end(ap);
}

// the bound of every host wait; 0 = not set yet (then the environment or the default)
static std::atomic<double> g_wait_limit{0.0};
double wait_limit_s()
{
	double v = g_wait_limit.load(std::memory_order_relaxed);
	if (v > 0) return v;
	const char* e = std::getenv("QPC_WAIT_LIMIT_S");
	char* end = nullptr;
	double x = e ? std::strtod(e, &end) : 0.0;
	v = (e && end != e && x > 0 && std::isfinite(x)) ? x : 600.0;
	double zero = 0.0;
	g_wait_limit.compare_exchange_strong(zero, v);
	return g_wait_limit.load(std::memory_order_relaxed);
}


// device status bits (never a trap)
enum : int { ST_PIVOT = 1, ST_NONFINITE = 2, ST_TIMEOUT = 4 };

// ============================================================================ kernels

// ---------------------------------------------------------------- layout change
// host layout [inst][m][l][r]  <->  engine layout [inst][m][r][l]
__global__ void k_to_rmajor(const double2* __restrict__ src, double2* __restrict__ dst, int N, int L, long nblk)
{
	long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	long tot = nblk * (long)N * L;
	if (t >= tot) return;
	long b = t / ((long)N * L);
	int rem = (int)(t % ((long)N * L));
	int r = rem / L, l = rem % L;
	dst[t] = src[b * (long)N * L + (long)l * N + r];
}
__global__ void k_to_lmajor(const double2* __restrict__ src, double2* __restrict__ dst, int N, int L, long nblk)
{
	long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	long tot = nblk * (long)N * L;
	if (t >= tot) return;
	long b = t / ((long)N * L);
	int rem = (int)(t % ((long)N * L));
	int l = rem / N, r = rem % N;
	dst[t] = src[b * (long)N * L + (long)r * L + l];
}

// ---------------------------------------------------------------- transform P (even/odd halves)
// Vh[m][kk][il]: row kk < npair = eigenvector of +s_kk, row npair = zero-eigenvalue vector.
// Eigen-basis slots per (inst,m,r) after the forward transform:
//   2k = z+_k = E_k + O_k,  2k+1 = conj(z-_k) = conj(E_k - O_k),  2*npair = Z (odd n_l)
// with E_k = sum_{il even} v_k[il] c[il], O_k = sum_{il odd} v_k[il] c[il], Z = sum_{il even} v_0[il] c[il].
// Backward (slots hold s_k = z+ + z-, d_k = z+ - z-, Z):
//   c[il even] = sum_k v_k[il] s_k + v_0[il] Z,  c[il odd] = sum_k v_k[il] d_k.
// One CTA = (inst, m, tile of TR rows); lane = row, warp = output unit; the
// row tile is staged in shared memory with an odd row stride (conflict-free
// 16-byte accesses).
constexpr int TR = 32;

__global__ void __launch_bounds__(256) k_transform(const double2* __restrict__ src, double2* __restrict__ dst,
	const double* __restrict__ Vh, int N, int L, int M, int npair, int forward,
	const int64_t* __restrict__ ntf, long step, int b0, int B, int cmode)
{
	// instances [b0, b0+B) of this launch (an instance group); cmode as in coupling_power
	extern __shared__ double2 sm[];
	const int ldt = L | 1;	// odd stride in 16-byte units
	double2* tin = sm;
	double2* tout = sm + TR * ldt;
	int tiles = (N + TR - 1) / TR;
	long blk = blockIdx.x;
	int tile = (int)(blk % tiles);
	long im_inst = (long)b0 * M + blk / tiles;
	int m = (int)(im_inst % M);
	long inst = im_inst / M;
	if (inst >= b0 + B) return;
	if (coupling_power(step, ntf[inst], cmode) == 0) return;
	int r0 = tile * TR;
	int nr = min(TR, N - r0);
	const double2* s = src + (im_inst * (long)N + r0) * L;
	double2* d = dst + (im_inst * (long)N + r0) * L;
	for (int t = threadIdx.x; t < nr * L; t += blockDim.x) {
		int rr = t / L, c = t % L;
		tin[rr * ldt + c] = s[t];
	}
	__syncthreads();
	const double* V = Vh + (long)m * (npair + 1) * L;
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	if (lane < nr) {
		const double2* row = tin + lane * ldt;
		if (forward) {
			const int nunit = npair + (L & 1);
			for (int u = warp; u < nunit; u += nw) {
				const double* v = V + (long)u * L;
				double er = 0.0, ei = 0.0, orr = 0.0, oi = 0.0;
				for (int il = 0; il < L; il += 2) {
					double w = v[il];
					double2 c = row[il];
					er = fma(w, c.x, er);
					ei = fma(w, c.y, ei);
				}
				if (u < npair) {
					for (int il = 1; il < L; il += 2) {
						double w = v[il];
						double2 c = row[il];
						orr = fma(w, c.x, orr);
						oi = fma(w, c.y, oi);
					}
					tout[lane * ldt + 2 * u] = make_double2(er + orr, ei + oi);
					tout[lane * ldt + 2 * u + 1] = make_double2(er - orr, oi - ei);
				} else {
					tout[lane * ldt + 2 * npair] = make_double2(er, ei);
				}
			}
		} else {
			for (int il = warp; il < L; il += nw) {
				int par = il & 1;
				double ar = 0.0, ai = 0.0;
				for (int k = 0; k < npair; ++k) {
					double w = V[(long)k * L + il];
					double2 c = row[2 * k + par];
					ar = fma(w, c.x, ar);
					ai = fma(w, c.y, ai);
				}
				if (!par && 2 * npair < L) {
					double w = V[(long)npair * L + il];
					double2 c = row[2 * npair];
					ar = fma(w, c.x, ar);
					ai = fma(w, c.y, ai);
				}
				tout[lane * ldt + il] = make_double2(ar, ai);
			}
		}
	}
	__syncthreads();
	for (int t = threadIdx.x; t < nr * L; t += blockDim.x) {
		int rr = t / L, c = t % L;
		d[t] = tout[rr * ldt + c];
	}
}

// ---------------------------------------------------------------- coupling factorisation
// LDL^T (no pivoting) of the complex-symmetric band S + i b R, b = lambda_k f(t_s) dt/4,
// for every (look-ahead step j, inst, m, pair k): one lane per system, the
// trailing (p+1)x(p+1) window of the right-looking elimination in registers.
// Output, row form per system: fac[sys][r][c], c < P: L(r, r-1-c); c = P: 1/D(r),
// sys = ((j*B + inst)*M + m)*npair + k.
template <int P>
__global__ void __launch_bounds__(64) k_factor(double2* __restrict__ fac, const double* __restrict__ S, const double* __restrict__ R,
	const double* __restrict__ lamp, const double* __restrict__ ftab, long ld, const int64_t* __restrict__ ntf,
	long step0, int K, int B, int b0, int Blive, int M, int N, int npair, double dt, int* __restrict__ status)
{
	constexpr int NE = P + 1;
	long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
	long nsys = (long)K * Blive * M * npair;
	if (g >= nsys) return;
	int k = (int)(g % npair);
	long t = g / npair;
	int m = (int)(t % M); t /= M;
	long inst = b0 + t % Blive;
	int j = (int)(t / Blive);
	long s = step0 + j;
	if (coupling_power(s, ntf[inst]) == 0) return;
	double f = ftab[inst * ld + s];
	double beta = lamp[m * npair + k] * ((f * (dt * 0.5)) * 0.5);
	double2* out = fac + ((((long)j * B + inst) * M + m) * npair + k) * (long)N * NE;
	double wr[NE][NE], wi[NE][NE];
#pragma unroll
	for (int a = 0; a < NE; ++a)
#pragma unroll
		for (int b = 0; b <= a; ++b) {
			// entry (a, b), b <= a: stored at S[b][a-b]
			wr[a][b] = __ldg(S + b * NE + (a - b));
			wi[a][b] = beta * __ldg(R + b * NE + (a - b));
		}
	int bad = 0;
	for (int i = 0; i < N; ++i) {
		double dr = wr[0][0], di = wi[0][0];
		double den = fma(dr, dr, di * di);
		if (!(den >= 1e-31)) bad = 1;
		double inv = 1.0 / den;
		double rr = dr * inv, ri = -di * inv;
		double lr[NE], li[NE];
		out[(long)i * NE + P] = make_double2(rr, ri);
#pragma unroll
		for (int a = 1; a < NE; ++a) {
			lr[a] = fma(wr[a][0], rr, -wi[a][0] * ri);
			li[a] = fma(wr[a][0], ri, wi[a][0] * rr);
			if (i + a < N) out[(long)(i + a) * NE + (a - 1)] = make_double2(lr[a], li[a]);
		}
		double cr[NE], ci[NE];	// column 0 before the update overwrites it
#pragma unroll
		for (int b = 1; b < NE; ++b) { cr[b] = wr[b][0]; ci[b] = wi[b][0]; }
#pragma unroll
		for (int a = 1; a < NE; ++a)
#pragma unroll
			for (int b = 1; b <= a; ++b) {
				// W[a-1][b-1] = W[a][b] - l_a * W[b][0]
				wr[a - 1][b - 1] = fma(-lr[a], cr[b], fma(li[a], ci[b], wr[a][b]));
				wi[a - 1][b - 1] = fma(-lr[a], ci[b], fma(-li[a], cr[b], wi[a][b]));
			}
		int rn = i + NE;
#pragma unroll
		for (int c = 0; c < NE; ++c) {
			int col = i + 1 + c;
			bool in = rn < N;
			wr[P][c] = in ? __ldg(S + (long)col * NE + (P - c)) : 0.0;
			wi[P][c] = in ? beta * __ldg(R + (long)col * NE + (P - c)) : 0.0;
		}
	}
	if (bad) atomicOr(status, ST_PIVOT);
}

// ---------------------------------------------------------------- reductions
// Per (inst, m, il) channel partial sums, then a fixed-order per-instance sum
// (deterministic: the same input gives bit-identical output).
__device__ __forceinline__ double2 band_sym_mv(const double* __restrict__ A, int NE, int N, const double2* __restrict__ x, long xs, int r)
{
	// (A x)_r for symmetric band A
	double re = 0.0, im = 0.0;
	for (int k = NE - 1; k >= 1; --k)
		if (r - k >= 0) { double a = __ldg(A + (long)(r - k) * NE + k); double2 v = x[(long)(r - k) * xs]; re = fma(a, v.x, re); im = fma(a, v.y, im); }
	for (int k = 0; k < NE && r + k < N; ++k) { double a = __ldg(A + (long)r * NE + k); double2 v = x[(long)(r + k) * xs]; re = fma(a, v.x, re); im = fma(a, v.y, im); }
	return make_double2(re, im);
}

// out[ch] = c^H A c' where c = channel ch, c' = channel ch + dl (same (inst,m)); zero if out of range
__global__ void k_band_inner(const double2* __restrict__ st, const double* __restrict__ A, int NE, int N, int L, long nch,
	int dl, double2* __restrict__ out)
{
	long ch = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (ch >= nch) return;
	int il = (int)(ch % L);
	int il2 = il + dl;
	if (il2 < 0 || il2 >= L) { out[ch] = make_double2(0.0, 0.0); return; }
	long base = (ch / L) * (long)N * L;
	const double2* x = st + base + il;
	const double2* y = st + base + il2;
	double re = 0.0, im = 0.0;
	for (int r = 0; r < N; ++r) {
		double2 t = band_sym_mv(A, NE, N, y, L, r);
		double2 c = x[(long)r * L];
		re = fma(c.x, t.x, fma(c.y, t.y, re));
		im = fma(c.x, t.y, fma(-c.y, t.x, im));
	}
	out[ch] = make_double2(re, im);
}

// proj[inst][m][il][n] = sum_r basis_l[n][r] c[r]
__global__ void k_projection(const double2* __restrict__ st, const double* __restrict__ basis, const long* __restrict__ boff,
	const int* __restrict__ nst, const long* __restrict__ poff, int N, int L, int M, int m0, long nch, int nmax,
	double2* __restrict__ proj)
{
	long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	long ch = t / nmax;
	int n = (int)(t % nmax);
	if (ch >= nch) return;
	int il = (int)(ch % L);
	int m = (int)((ch / L) % M) + m0;
	int l = il + (m < 0 ? -m : m);
	if (n >= nst[l]) return;
	const double* b = basis + boff[l] + (long)n * N;
	const double2* x = st + (ch / L) * (long)N * L + il;
	double re = 0.0, im = 0.0;
	for (int r = 0; r < N; ++r) { double w = __ldg(b + r); double2 c = x[(long)r * L]; re = fma(w, c.x, re); im = fma(w, c.y, im); }
	proj[poff[ch] + n] = make_double2(re, im);
}

// In-loop dipole, l basis: per channel of instances with nt_field <= step < nt_total,
// dl = 2 y10(m,il) Re <c_il|F|c_il+1>  (observable_z::observe, observable/1e.hpp:26-50)
__global__ void k_dipole_lbasis(const double2* __restrict__ st, const double* __restrict__ F, const double* __restrict__ y10,
	const int64_t* __restrict__ ntf, const int64_t* __restrict__ ntt, long step, int b0, int cnt, int M, int N, int L, int NE,
	double* __restrict__ dl)
{
	long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= (long)cnt * M * L) return;
	long ch = (long)b0 * M * L + t;
	int il = (int)(ch % L);
	long im_inst = ch / L;
	int m = (int)(im_inst % M);
	long inst = im_inst / M;
	if (!(step >= ntf[inst] && step < ntt[inst])) return;
	double v = 0.0;
	if (il + 1 < L) {
		const double2* x = st + im_inst * (long)N * L + il;
		const double2* y = x + 1;
		double re = 0.0;
		for (int r = 0; r < N; ++r) {
			double tr = 0.0, ti = 0.0;
			for (int k = NE - 1; k >= 1; --k)
				if (r - k >= 0) { double a = __ldg(F + (long)(r - k) * NE + k); double2 w = y[(long)(r - k) * L]; tr = fma(a, w.x, tr); ti = fma(a, w.y, ti); }
			for (int k = 0; k < NE && r + k < N; ++k) { double a = __ldg(F + (long)r * NE + k); double2 w = y[(long)(r + k) * L]; tr = fma(a, w.x, tr); ti = fma(a, w.y, ti); }
			double2 c = x[(long)r * L];
			re = fma(c.x, tr, fma(c.y, ti, re));
		}
		v = 2.0 * y10[m * L + il] * re;
	}
	dl[ch] = v;
}

// Per instance of [b0, b0+cnt) with step < nt_total: the dipole at t_step, from the
// eigen-basis observation of the coupling chains (sum_k s_k (<z+|F|z+> - <z-|F|z->))
// while the instance is in its pulse, from the l-basis terms otherwise; fixed
// summation order.
__global__ void k_dipole_combine(const double* __restrict__ obs, const double* __restrict__ dl, const double* __restrict__ lamp,
	const int64_t* __restrict__ ntf, const int64_t* __restrict__ ntt, long step, int b0, int cnt, int M, int L, int np,
	double* __restrict__ zdev, long ldz)
{
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= cnt) return;
	long inst = b0 + t;
	if (step >= ntt[inst] && !(ntf[inst] > 0 && step < ntf[inst])) return;
	double v = 0.0;
	if (ntf[inst] > 0 && step < ntf[inst]) {
		for (int m = 0; m < M; ++m)
			for (int k = 0; k < np; ++k) {
				long c = ((inst * M + m) * np + k) * 2;
				v += lamp[m * np + k] * (obs[c] - obs[c + 1]);
			}
	} else {
		for (long c = inst * M * L; c < (inst + 1) * M * L; ++c) v += dl[c];
	}
	zdev[inst * ldz + step] = v;
}

__global__ void k_status_check(const double2* __restrict__ st, long n, int* __restrict__ status)
{
	long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= n) return;
	double2 v = st[t];
	if (!isfinite(v.x) || !isfinite(v.y)) atomicOr(status, ST_NONFINITE);
}

} // namespace qpc

using namespace qpc;

// ============================================================================ handle

// chain-kernel choice meaning "the segmented solver" (k_chain_seg); 0 in gsel means "not tuned yet"
constexpr int QPC_SEG = -1;

struct qpc_lgwz {
	int dev = 0;
	qpc_dims d{};
	int N = 0, P = 0, L = 0, M = 0, B = 0, lmax = 0, nlh = 0, npair = 0;
	double dt = 0.0;
	cudaStream_t stream = nullptr;
	cudaEvent_t ev0 = nullptr, ev1 = nullptr;	// brackets of qpc_lgwz_run
	cudaEvent_t evt0 = nullptr, evt1 = nullptr;	// autotuner timing
	// instance groups advance on their own streams, so that the kernels of one
	// group fill the FP64 pipes the other group leaves idle
	static constexpr int MAXNS = 4;
	int NS = 1;
	cudaStream_t gs[MAXNS] = {nullptr, nullptr, nullptr, nullptr};
	cudaEvent_t gev[MAXNS] = {nullptr, nullptr, nullptr, nullptr};
	cudaEvent_t xev = nullptr;	// main stream -> instance groups, after the per-step extras of a run
	int* slotmap = nullptr;		// device [B]: the sorted slot of each instance during a run (t-SURFF)
	double* S = nullptr;      // [N][P+1]
	double* R = nullptr;      // [N][P+1]
	double* Vh = nullptr;     // [M][npair+1][L]
	double* lamp = nullptr;   // [M][npair]
	double2* ff = nullptr;    // field-free factors [nlh][N][P+1] (row form + 1/D); [B][nlh][N][P+1] with hpi
	int hpi = 0;              // one Hamiltonian (potential) per instance
	// segmented chain solver (k_chain_seg) for handles with few wavefunctions: Q segments of Ls rows and
	// the spikes [block][N][P] of the coupling factors (per look-ahead slot) and of the field-free ones
	bool seg_ok = false;
	int Q = 1, Ls = 0;
	int cmode = 0;	// coupling mode of the launches being enqueued (coupling_power): 0 fused, 1 closing, 2 opening
	bool seg_sfac[2] = {false, false};	// [coupling]: the factor block staged in shared memory
	size_t seg_smem[2] = {0, 0};		// [coupling]: dynamic shared memory of k_chain_seg
	double2 *spf_c = nullptr, *spb_c = nullptr, *spf_ff = nullptr, *spb_ff = nullptr;
	int* ffmap = nullptr;     // device [B]: the instance whose factors a (sorted) instance uses, during a run
	int* ffmap_id = nullptr;  // device [B]: identity
	const int* ffmap_cur = nullptr;	// ffmap during a run, ffmap_id otherwise (NULL without hpi)
	double2* st = nullptr;    // state, engine layout [B][M][N][L]
	double2* eo = nullptr;    // eigen-basis state [B][M][N][L]
	double2* wk = nullptr;    // per-chain work vector [B][M][N][L]
	double2* hostlay = nullptr; // [B][M][L][N] staging for layout changes
	double2* fac = nullptr;   // coupling factors [K][B][M][npair][N][P+1]
	int K = 1;
	int* status = nullptr;
	double2* red = nullptr;   // reduction scratch [2*B*M*L]
	// absorbing mask: the mask band and the Cholesky factor of S (set by qpc_lgwz_mask)
	double *mM = nullptr, *mLrow = nullptr, *mLcol = nullptr, *mdinv = nullptr;
	// in-loop dipole (qpc_lgwz_run_dipole)
	double* obsF = nullptr;   // device band of <B|f|B> [N][P+1]
	double* obs = nullptr;    // per coupling chain [B][M][npair][2]
	double* dl = nullptr;     // per channel [B][M][L]
	double* y10d = nullptr;   // [M][L]
	double* zdev = nullptr;   // [B][ldz]
	size_t zcap = 0;
	long ldz = 0;
	bool observing = false;
	int64_t* ntf = nullptr;   // device [B]
	int64_t* ntt = nullptr;
	double* ftab = nullptr;   // device field table [B][ld]
	size_t ftab_cap = 0;
	long ld = 1;
	double last_ms = 0.0;
	int64_t launches = 0;
	// chain-kernel lanes per part chosen by the autotuner, per (coupling?, live-instance bucket)
	int gsel[2][32];
	std::vector<int> gcand;
	size_t chain_smem = 0;
	int chain_sstage = 1;	// k_chain stages the S band in shared memory (QPC_CHAIN_SSTAGE=0: read through L1)
	int chain_warps = 4;	// warps per k_chain block, sharing one staged S band (QPC_CHAIN_WARPS)
	// the l-space transforms on the tensor cores (qpc_ltrans.cu) for n_l <= 48: half-width of the
	// block-diagonal product (0: the FP64 kernel k_transform only), the matrices' digit planes
	// [M][2][8][2 lt_kb][64] and exponents [M][2][2 lt_kb].  A launch uses them when it has at least
	// one 64-row tile per SM (lt_min_tiles; measured: with fewer, as for one wavefunction, the FP64
	// kernel's shorter latency wins); QPC_LTRANS_TC=1 uses them for every launch, 0 for none.
	int lt_kb = 0;
	long lt_min_tiles = 0;
	bool lt_failed = false;	// a transform launch could not be enqueued (reported by read_status)
	uint16_t* lt_dig = nullptr;
	int* lt_fex = nullptr;
	// optional per-kernel timing (CUDA events around each launch on the handle's stream)
	bool profiling = false;
	std::vector<cudaEvent_t> evpool;
	std::vector<std::pair<int, int>> evuse;	// (kernel id, index of start event; end = +1)
	double kms[QPC_NKERNEL] = {0};
	int64_t kcount[QPC_NKERNEL] = {0};
	std::vector<double> h_lam;   // [M][L]
	std::vector<double> h_P;     // [M][L][L]
};

// ---------------------------------------------------------------- absorbing mask
// absorber_mask::operator() (absorber.hpp:51-63) on the engine's r-major state [B][M][N][L]:
// t = M c per channel (all lanes, one element each), then c = (L L^T)^-1 t with one lane per
// real recurrence (channel, real or imaginary part); Lrow[r][j-1] = L(r, r-j),
// Lcol[r][k-1] = L(r+k, r), dinv[r] = 1/L(r, r).
// mask_active: inside a run, the instance (sorted slot) takes the mask after loop step s - 1 when
// 1 <= s <= nt_total (ntt == NULL: every instance, the stand-alone call)
__device__ __forceinline__ bool mask_active(const int64_t* __restrict__ ntt, long step, long inst)
{
	return !ntt || (step >= 1 && step <= ntt[inst]);
}

__global__ void k_mask_band(const double2* __restrict__ st, double2* __restrict__ t, const double* __restrict__ Mb, int N, int P, int L,
	long total, const int64_t* __restrict__ ntt = nullptr, long step = 0, long per_inst = 1)
{
	const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= total) return;
	if (!mask_active(ntt, step, e / per_inst)) return;
	const long row = e / L;
	const int r = (int)(row % N);
	double2 acc = make_double2(0.0, 0.0);
	for (int q = 1; q <= P && q <= r; ++q) {
		double m = Mb[(long)(r - q) * (P + 1) + q];
		double2 v = st[e - (long)q * L];
		acc.x = fma(m, v.x, acc.x); acc.y = fma(m, v.y, acc.y);
	}
	for (int q = 0; q <= P && r + q < N; ++q) {
		double m = Mb[(long)r * (P + 1) + q];
		double2 v = st[e + (long)q * L];
		acc.x = fma(m, v.x, acc.x); acc.y = fma(m, v.y, acc.y);
	}
	t[e] = acc;
}

template <int P>
__global__ void k_mask_solve(double2* __restrict__ st, double2* __restrict__ tb, const double* __restrict__ Lrow,
	const double* __restrict__ Lcol, const double* __restrict__ dinv, int N, int L, long nchain,
	const int64_t* __restrict__ ntt = nullptr, long step = 0, int M = 1)
{
	const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (c >= nchain) return;
	const long bm = c / (2L * L);
	if (!mask_active(ntt, step, bm / M)) return;
	const int rest = (int)(c - bm * 2L * L);	// l * 2 + part
	const long stride = 2L * L;
	double* t = reinterpret_cast<double*>(tb) + bm * N * stride + rest;
	double* x = reinterpret_cast<double*>(st) + bm * N * stride + rest;
	double w[P];
#pragma unroll
	for (int j = 0; j < P; ++j) w[j] = 0.0;
	for (int r = 0; r < N; ++r) {
		double v = t[(long)r * stride];
#pragma unroll
		for (int j = 0; j < P; ++j) v = fma(-w[j], Lrow[(long)r * P + j], v);
		v *= dinv[r];
#pragma unroll
		for (int j = P - 1; j > 0; --j) w[j] = w[j - 1];
		w[0] = v;
		t[(long)r * stride] = v;
	}
#pragma unroll
	for (int j = 0; j < P; ++j) w[j] = 0.0;
	for (int r = N - 1; r >= 0; --r) {
		double v = t[(long)r * stride];
#pragma unroll
		for (int j = 0; j < P; ++j) v = fma(-w[j], Lcol[(long)r * P + j], v);
		v *= dinv[r];
#pragma unroll
		for (int j = P - 1; j > 0; --j) w[j] = w[j - 1];
		w[0] = v;
		x[(long)r * stride] = v;
	}
}

namespace {

long state_len(const qpc_lgwz* h) { return (long)h->B * h->M * h->N * h->L; }

int wait_stream(qpc_lgwz* h) { return wait_on(h->stream); }

int read_status(qpc_lgwz* h)
{
	int st = 0;
	if (int rc = copy_to_host(&st, h->status, sizeof(int), h->stream)) return rc;
	if (h->lt_failed) {
		h->lt_failed = false;
		set_error("an l-space transform launch could not be enqueued");
		return QPC_ERR_CUDA;
	}
	if (st & ST_PIVOT) { set_error("zero pivot in a Crank-Nicolson factorisation"); return QPC_ERR_SINGULAR; }
	if (st & ST_NONFINITE) { set_error("non-finite value in the state"); return QPC_ERR_NUMERIC; }
	if (st & ST_TIMEOUT) { set_error("a tensor-core wait of the l-space transform ran out"); return QPC_ERR_TIMEOUT; }
	return QPC_OK;
}

#define LAUNCH(h) ((h)->launches++)

struct prof_scope {
	qpc_lgwz* h; int kind; cudaStream_t st; int idx = -1;
	prof_scope(qpc_lgwz* h_, int kind_, cudaStream_t st_) : h(h_), kind(kind_), st(st_)
	{
		if (!h->profiling) return;
		idx = (int)h->evuse.size() * 2;
		while ((int)h->evpool.size() < idx + 2) { cudaEvent_t e; cudaEventCreate(&e); h->evpool.push_back(e); }
		cudaEventRecord(h->evpool[idx], st);
	}
	~prof_scope()
	{
		if (idx < 0) return;
		cudaEventRecord(h->evpool[idx + 1], st);
		h->evuse.push_back({kind, idx});
	}
};

void collect_profile(qpc_lgwz* h)
{
	for (auto& u : h->evuse) {
		float ms = 0.f;
		if (cudaEventElapsedTime(&ms, h->evpool[u.second], h->evpool[u.second + 1]) == cudaSuccess) {
			h->kms[u.first] += ms;
			h->kcount[u.first] += 1;
		}
	}
	h->evuse.clear();
}

// ---------------------------------------------------------------- chain launches
template <int P, int G, bool CPL>
void launch_chain_g(qpc_lgwz* h, cudaStream_t st, int b0, double2* X, const double2* fac, const int64_t* nta, long step, int jslot, int cnt)
{
	using C = chain_cfg<P, G, CPL>;
	long per = CPL ? (long)h->M * h->npair * 2 : (long)h->M * h->L;
	long nch = (long)cnt * per;
	if (nch <= 0) return;
	long chbase = (long)b0 * per;
	long nwarps = (nch + C::CPW - 1) / C::CPW;
	const int wpb = h->chain_warps;
	unsigned grid = (unsigned)((nwarps + wpb - 1) / wpb);
	bool ob = CPL && h->observing;
	k_chain<P, G, CPL><<<grid, 32 * wpb, h->chain_sstage ? h->chain_smem : 0, st>>>(X, h->wk, fac, h->S, nta, step, jslot, h->B, h->M,
		h->d.m0, h->N, h->L, h->npair, chbase, chbase + nch, ob ? h->obsF : nullptr, ob ? h->obs : nullptr,
		CPL ? nullptr : h->ffmap_cur, (long)h->nlh * h->N * (h->P + 1), h->cmode, h->chain_sstage);
	LAUNCH(h);
}

template <int P, bool CPL>
void launch_chain_seg(qpc_lgwz* h, cudaStream_t st, int b0, double2* X, const double2* fac, const int64_t* nta, long step, int jslot, int cnt)
{
	long per = CPL ? (long)h->M * h->npair * 2 : (long)h->M * h->L;
	long nch = (long)cnt * per;
	if (nch <= 0) return;
	long chbase = (long)b0 * per;
	unsigned grid = (unsigned)(nch / (CPL ? 2 : 1));
	const size_t smem = h->seg_smem[CPL];
	if (h->seg_sfac[CPL])
		k_chain_seg<P, CPL, true><<<grid, SEG_THREADS, smem, st>>>(X, fac, CPL ? h->spf_c : h->spf_ff, CPL ? h->spb_c : h->spb_ff, h->S, nta, step,
			jslot, h->B, h->M, h->d.m0, h->N, h->L, h->npair, chbase, chbase + nch, h->Q, h->Ls, CPL ? nullptr : h->ffmap_cur,
			(long)h->nlh * h->N * (h->P + 1), h->cmode);
	else
		k_chain_seg<P, CPL, false><<<grid, SEG_THREADS, smem, st>>>(X, fac, CPL ? h->spf_c : h->spf_ff, CPL ? h->spb_c : h->spb_ff, h->S, nta, step,
			jslot, h->B, h->M, h->d.m0, h->N, h->L, h->npair, chbase, chbase + nch, h->Q, h->Ls, CPL ? nullptr : h->ffmap_cur,
			(long)h->nlh * h->N * (h->P + 1), h->cmode);
	LAUNCH(h);
}

template <int P, bool CPL>
void launch_chain(qpc_lgwz* h, cudaStream_t st, int b0, int G, double2* X, const double2* fac, const int64_t* nta, long step, int jslot, int cnt)
{
	// G = QPC_SEG (-1): the segmented solver; it has no observation pass, so an observed coupling step uses G = P
	if (G == QPC_SEG && (!h->seg_ok || (CPL && h->observing))) G = P;
	switch (G) {
	case QPC_SEG: launch_chain_seg<P, CPL>(h, st, b0, X, fac, nta, step, jslot, cnt); break;
	case 1: launch_chain_g<P, 1, CPL>(h, st, b0, X, fac, nta, step, jslot, cnt); break;
	case 2: if constexpr (P % 2 == 0) launch_chain_g<P, 2, CPL>(h, st, b0, X, fac, nta, step, jslot, cnt); break;
	case 3: if constexpr (P % 3 == 0) launch_chain_g<P, 3, CPL>(h, st, b0, X, fac, nta, step, jslot, cnt); break;
	case 4: if constexpr (P % 4 == 0) launch_chain_g<P, 4, CPL>(h, st, b0, X, fac, nta, step, jslot, cnt); break;
	default: launch_chain_g<P, P, CPL>(h, st, b0, X, fac, nta, step, jslot, cnt); break;
	}
}

template <int P>
void set_chain_smem_attr(size_t smem)
{
	auto f = [&](auto kern) { cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); };
	f(k_chain<P, 1, true>); f(k_chain<P, 1, false>); f(k_chain<P, P, true>); f(k_chain<P, P, false>);
	if constexpr (P % 2 == 0) { f(k_chain<P, 2, true>); f(k_chain<P, 2, false>); }
	if constexpr (P % 3 == 0) { f(k_chain<P, 3, true>); f(k_chain<P, 3, false>); }
	if constexpr (P % 4 == 0) { f(k_chain<P, 4, true>); f(k_chain<P, 4, false>); }
}

int live_bucket(int n) { int b = 0; while ((1 << b) < n) ++b; return b; }

// Autotuner: for the current live-instance count, time every candidate G for
// the coupling and the field-free chain kernels (two launches each, CUDA
// events) on scratch buffers (eo / wk / the factor slot of this step, whose
// contents are about to be overwritten) and keep the fastest.  Runs before
// the step's forward transform, once per (kernel, live bucket).
// Tuning decisions are shared by every handle of the process with the same grid shape, so that
// two handles that do the same work choose the same kernels and give bit-identical results (the
// candidates differ in rounding); the first handle to meet a (shape, live bucket) times it.
std::mutex g_tune_mu;
std::map<std::vector<long>, int> g_tune;

std::vector<long> tune_key(const qpc_lgwz* h, int cpl, int bk)
{
	return {h->dev, h->N, h->P, h->L, h->M, h->npair, h->NS, h->hpi, h->seg_ok ? 1 : 0, cpl, bk};
}

template <int P>
int autotune_one(qpc_lgwz* h, int cpl, long step, int jslot, int Bl)
{
	int bk = live_bucket(Bl);
	if (Bl <= 0 || h->gsel[cpl][bk]) return QPC_OK;
	// QPC_CHAIN_G fixes the lanes per part instead (a candidate that divides P, or -1 for the segmented solver)
	if (const char* e = getenv("QPC_CHAIN_G")) {
		const int G = atoi(e);
		if (std::find(h->gcand.begin(), h->gcand.end(), G) != h->gcand.end()) { h->gsel[cpl][bk] = G; return QPC_OK; }
	}
	{
		std::lock_guard<std::mutex> lk(g_tune_mu);
		auto it = g_tune.find(tune_key(h, cpl, bk));
		if (it != g_tune.end()) { h->gsel[cpl][bk] = it->second; return QPC_OK; }
	}
	float best = 1e30f;
	int bestg = 1;
	const bool obs_saved = h->observing;
	h->observing = false;	// trials write nothing but scratch
	struct restore { qpc_lgwz* h; bool v; ~restore() { h->observing = v; } } rs{h, obs_saved};
	for (int G : h->gcand) {
		float tot = 0.f;
		for (int rep = 0; rep < 2; ++rep) {
			QPC_CUDA(cudaEventRecord(h->evt0, h->stream));
			if (cpl) launch_chain<P, true>(h, h->stream, 0, G, h->eo, h->fac, h->ntf, step, jslot, Bl);
			else launch_chain<P, false>(h, h->stream, 0, G, h->eo, h->ff, h->ntt, step, 0, Bl);
			QPC_CUDA(cudaEventRecord(h->evt1, h->stream));
			if (int rc = wait_stream(h)) return rc;
			float ms = 0.f;
			cudaEventElapsedTime(&ms, h->evt0, h->evt1);
			if (rep) tot += ms;
		}
		QPC_CUDA(cudaGetLastError());
		if (tot < best) { best = tot; bestg = G; }
	}
	std::lock_guard<std::mutex> lk(g_tune_mu);
	auto ins = g_tune.emplace(tune_key(h, cpl, bk), bestg);	// a handle tuning concurrently may have stored first
	h->gsel[cpl][bk] = ins.first->second;
	return QPC_OK;
}

// Autotuner: for a live-instance count not seen before, time every candidate G
// of the coupling and the field-free chain kernels (two launches each, CUDA
// events) on scratch buffers (eo, wk and this step's factor slot, whose
// contents are overwritten before use) and keep the fastest.  Runs with all
// group streams idle, before the step's forward transforms.
template <int P>
int autotune(qpc_lgwz* h, long step, int jslot, const int* Bc, const int* Bf)
{
	bool need = false;
	for (int g = 0; g < h->NS; ++g) {
		if (Bc[g] > 0 && h->npair > 0 && !h->gsel[1][live_bucket(Bc[g])]) need = true;
		if (Bf[g] > 0 && !h->gsel[0][live_bucket(Bf[g])]) need = true;
	}
	if (!need) return QPC_OK;
	for (int g = 0; g < h->NS; ++g)
		if (int rc = wait_on(h->gs[g])) return rc;
	for (int g = 0; g < h->NS; ++g) {
		if (h->npair > 0) if (int rc = autotune_one<P>(h, 1, step, jslot, Bc[g])) return rc;
		if (int rc = autotune_one<P>(h, 0, step, jslot, Bf[g])) return rc;
	}
	return QPC_OK;
}

// All kernels of loop index `step` for the instance group [b0, b0+...) on stream st:
// Bc instances in their pulse (coupling), Bf with field-free work, factor look-ahead
// for Bfac instances when do_factor.
template <int P>
void launch_group_step(qpc_lgwz* h, cudaStream_t st, int b0, long step, long step0, int jslot, bool do_factor, int kfac,
	int Bc, int Bf, int Bfac)
{
	const int B = h->B, M = h->M, N = h->N, L = h->L, np = h->npair;
	if (do_factor && np > 0 && Bfac > 0) {
		prof_scope ps(h, QPC_KERNEL_FACTOR, st);
		long nsys = (long)kfac * Bfac * M * np;
		k_factor<P><<<(unsigned)((nsys + 63) / 64), 64, 0, st>>>(h->fac, h->S, h->R, h->lamp, h->ftab, h->ld,
			h->ntf, step0, kfac, B, b0, Bfac, M, N, np, h->dt, h->status);
		LAUNCH(h);
		if (h->seg_ok) {
			const long total = (long)kfac * Bfac * M * np * h->Q * P * 2;
			k_spikes<P><<<(unsigned)((total + 127) / 128), 128, 0, st>>>(h->fac, h->spf_c, h->spb_c, B, b0, Bfac, M, np, N, h->Q, h->Ls, total);
			LAUNCH(h);
		}
	}
	if (Bc > 0 && (np > 0 || (L & 1))) {
		int tiles = (N + TR - 1) / TR;
		size_t smem = sizeof(double2) * 2 * TR * (L | 1);
		unsigned grid = (unsigned)((long)Bc * M * tiles);
		const bool use_tc = h->lt_kb && (long)Bc * M * ((N + 63) / 64) >= h->lt_min_tiles;
		{
			prof_scope ps(h, QPC_KERNEL_TRANSFORM_FWD, st);
			if (use_tc) {
				if (ltrans_launch(h->lt_kb, h->st, h->eo, h->lt_dig, h->lt_fex, N, L, M, np, 1, h->ntf, step, b0, Bc, h->cmode, h->status,
						ST_TIMEOUT, st))
					h->lt_failed = true;
			} else
				k_transform<<<grid, 256, smem, st>>>(h->st, h->eo, h->Vh, N, L, M, np, 1, h->ntf, step, b0, Bc, h->cmode);
			LAUNCH(h);
		}
		if (np > 0) {
			prof_scope ps(h, QPC_KERNEL_SWEEP, st);
			launch_chain<P, true>(h, st, b0, h->gsel[1][live_bucket(Bc)], h->eo, h->fac, h->ntf, step, jslot, Bc);
		}
		{
			prof_scope ps(h, QPC_KERNEL_TRANSFORM_BWD, st);
			if (use_tc) {
				if (ltrans_launch(h->lt_kb, h->eo, h->st, h->lt_dig, h->lt_fex, N, L, M, np, 0, h->ntf, step, b0, Bc, h->cmode, h->status,
						ST_TIMEOUT, st))
					h->lt_failed = true;
			} else
				k_transform<<<grid, 256, smem, st>>>(h->eo, h->st, h->Vh, N, L, M, np, 0, h->ntf, step, b0, Bc, h->cmode);
			LAUNCH(h);
		}
	}
	if (h->observing) {
		// the dipole at t_step of every instance with step < nt_total (before its field-free step)
		int cnt = std::max(Bc, Bf);
		if (cnt > 0) {
			long nch = (long)cnt * M * L;
			k_dipole_lbasis<<<(unsigned)((nch + 127) / 128), 128, 0, st>>>(h->st, h->obsF, h->y10d, h->ntf, h->ntt, step, b0, cnt,
				M, N, L, h->P + 1, h->dl);
			k_dipole_combine<<<(unsigned)((cnt + 127) / 128), 128, 0, st>>>(h->obs, h->dl, h->lamp, h->ntf, h->ntt, step, b0, cnt,
				M, L, np, h->zdev, h->ldz);
			h->launches += 2;
		}
	}
	if (Bf > 0) {
		prof_scope ps(h, QPC_KERNEL_FIELDFREE, st);
		launch_chain<P, false>(h, st, b0, h->gsel[0][live_bucket(Bf)], h->st, h->ff, h->ntt, step, 0, Bf);
	}
}

template <int P>
int launch_step_t(qpc_lgwz* h, long step, long step0, int jslot, bool do_factor, int kfac, const int* gb,
	const int* Bc, const int* Bf)
{
	if (int rc = autotune<P>(h, step, jslot, Bc, Bf)) return rc;
	for (int g = 0; g < h->NS; ++g)
		launch_group_step<P>(h, h->gs[g], gb[g], step, step0, jslot, do_factor, kfac, Bc[g], Bf[g], Bc[g]);
	return QPC_OK;
}

// What a run does to the state between two steps (the driver loop's t-SURFF accumulate and
// absorbing mask after each propagate, binsrc/sphTDSE.cpp:800-810), enqueued on the main stream
// once the instance groups have finished the closing half: fn(step) for loop step `step`.
struct between_steps {
	std::function<int(long)> fn;
};

// Loop step s of a run with work between steps: every coupling step is split in its closing half
// (the end of step s - 1) and its opening half (step s), with the extras in between; the factors
// of f(t_s) serve both halves.
template <int P>
int launch_split_t(qpc_lgwz* h, long step, long step0, int jslot, bool do_factor, int kfac, const int* gb, const int* Bc, const int* Bf,
	const between_steps& x)
{
	if (int rc = autotune<P>(h, step, jslot, Bc, Bf)) return rc;
	bool fac = do_factor;
	if (step > 0) {
		h->cmode = 1;
		for (int g = 0; g < h->NS; ++g) launch_group_step<P>(h, h->gs[g], gb[g], step, step0, jslot, fac, kfac, Bc[g], 0, Bc[g]);
		h->cmode = 0;
		fac = false;
		for (int g = 0; g < h->NS; ++g) {
			QPC_CUDA(cudaEventRecord(h->gev[g], h->gs[g]));
			QPC_CUDA(cudaStreamWaitEvent(h->stream, h->gev[g], 0));
		}
		if (int rc = x.fn(step)) return rc;
		QPC_CUDA(cudaEventRecord(h->xev, h->stream));
		for (int g = 0; g < h->NS; ++g) QPC_CUDA(cudaStreamWaitEvent(h->gs[g], h->xev, 0));
	}
	h->cmode = 2;
	for (int g = 0; g < h->NS; ++g) launch_group_step<P>(h, h->gs[g], gb[g], step, step0, jslot, fac, kfac, Bc[g], Bf[g], Bc[g]);
	h->cmode = 0;
	return QPC_OK;
}

int launch_split(qpc_lgwz* h, long step, long step0, int jslot, bool do_factor, int kfac, const int* gb, const int* Bc, const int* Bf,
	const between_steps& x)
{
	switch (h->P) {
	case 3: return launch_split_t<3>(h, step, step0, jslot, do_factor, kfac, gb, Bc, Bf, x);
	case 4: return launch_split_t<4>(h, step, step0, jslot, do_factor, kfac, gb, Bc, Bf, x);
	case 5: return launch_split_t<5>(h, step, step0, jslot, do_factor, kfac, gb, Bc, Bf, x);
	case 6: return launch_split_t<6>(h, step, step0, jslot, do_factor, kfac, gb, Bc, Bf, x);
	case 7: return launch_split_t<7>(h, step, step0, jslot, do_factor, kfac, gb, Bc, Bf, x);
	case 8: return launch_split_t<8>(h, step, step0, jslot, do_factor, kfac, gb, Bc, Bf, x);
	default: set_error("unsupported B-spline degree %d", h->P); return QPC_ERR_ARGS;
	}
}

int launch_step(qpc_lgwz* h, long step, long step0, int jslot, bool do_factor, int kfac, const int* gb, const int* Bc, const int* Bf)
{
	switch (h->P) {
	case 3: return launch_step_t<3>(h, step, step0, jslot, do_factor, kfac, gb, Bc, Bf);
	case 4: return launch_step_t<4>(h, step, step0, jslot, do_factor, kfac, gb, Bc, Bf);
	case 5: return launch_step_t<5>(h, step, step0, jslot, do_factor, kfac, gb, Bc, Bf);
	case 6: return launch_step_t<6>(h, step, step0, jslot, do_factor, kfac, gb, Bc, Bf);
	case 7: return launch_step_t<7>(h, step, step0, jslot, do_factor, kfac, gb, Bc, Bf);
	case 8: return launch_step_t<8>(h, step, step0, jslot, do_factor, kfac, gb, Bc, Bf);
	default: set_error("unsupported B-spline degree %d", h->P); return QPC_ERR_ARGS;
	}
}

// The dynamic shared-memory limit is a property of the kernel on a device, shared by
// every handle: it only ever grows, to the largest size any handle on that device needs.
std::mutex g_attr_mu;
std::map<std::pair<int, int>, size_t> g_attr_max;	// (device, kernel family) -> limit set

bool raise_attr(int dev, int family, size_t smem)
{
	std::lock_guard<std::mutex> lk(g_attr_mu);
	size_t& cur = g_attr_max[{dev, family}];
	if (smem <= cur) return false;
	cur = smem;
	return true;
}

template <int P>
void set_seg_smem_attr(qpc_lgwz* h)
{
	for (int cpl = 0; cpl < 2; ++cpl) {
		const size_t smem = h->seg_smem[cpl];
		if (smem <= 48 * 1024 || !raise_attr(h->dev, 100 + 4 * P + 2 * cpl + (h->seg_sfac[cpl] ? 1 : 0), smem)) continue;
		if (cpl && h->seg_sfac[1]) cudaFuncSetAttribute(k_chain_seg<P, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (cpl && !h->seg_sfac[1]) cudaFuncSetAttribute(k_chain_seg<P, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (!cpl && h->seg_sfac[0]) cudaFuncSetAttribute(k_chain_seg<P, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (!cpl && !h->seg_sfac[0]) cudaFuncSetAttribute(k_chain_seg<P, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	}
}

void set_smem_attrs(qpc_lgwz* h, size_t tr_smem)
{
	if (tr_smem > 48 * 1024 && raise_attr(h->dev, 0, tr_smem))
		cudaFuncSetAttribute(k_transform, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tr_smem);
	if (h->seg_ok) {
		switch (h->P) {
		case 3: set_seg_smem_attr<3>(h); break;
		case 4: set_seg_smem_attr<4>(h); break;
		case 5: set_seg_smem_attr<5>(h); break;
		case 6: set_seg_smem_attr<6>(h); break;
		case 7: set_seg_smem_attr<7>(h); break;
		case 8: set_seg_smem_attr<8>(h); break;
		}
	}
	if (!raise_attr(h->dev, h->P, h->chain_smem)) return;
	switch (h->P) {
	case 3: set_chain_smem_attr<3>(h->chain_smem); break;
	case 4: set_chain_smem_attr<4>(h->chain_smem); break;
	case 5: set_chain_smem_attr<5>(h->chain_smem); break;
	case 6: set_chain_smem_attr<6>(h->chain_smem); break;
	case 7: set_chain_smem_attr<7>(h->chain_smem); break;
	case 8: set_chain_smem_attr<8>(h->chain_smem); break;
	}
}

// reorder instances on the device: dst[k] = src[perm[k]] (whole instance blocks)
int permute_instances(qpc_lgwz* h, const std::vector<int>& perm, bool inverse)
{
	size_t blk = sizeof(double2) * (size_t)h->M * h->N * h->L;
	for (int k = 0; k < h->B; ++k) {
		int from = inverse ? k : perm[k], to = inverse ? perm[k] : k;
		QPC_CUDA(cudaMemcpyAsync((char*)h->eo + blk * to, (const char*)h->st + blk * from, blk, cudaMemcpyDeviceToDevice, h->stream));
	}
	std::swap(h->st, h->eo);
	return QPC_OK;
}

} // namespace

// spikes of nblk field-free factor blocks (row form [blk][N][P+1]) for the segmented solver
template <int P>
static void host_spikes(const double2* fac, size_t nblk, int N, int Q, int Ls, double2* sf, double2* sb)
{
	for (size_t bl = 0; bl < nblk; ++bl)
		for (int sg = 0; sg < Q; ++sg) {
			const int a = sg * Ls, b = std::min(N, a + Ls);
			for (int j = 1; j <= P; ++j) {
				seg_spike<P>(fac + bl * N * (P + 1), N, a, b, j, true, sf + bl * N * P);
				seg_spike<P>(fac + bl * N * (P + 1), N, a, b, j, false, sb + bl * N * P);
			}
		}
}

extern "C" {

const char* qpc_last_error(void) { return g_err; }

// FP64 FMA throughput probe: every thread advances 8 independent chains of dependent DFMAs
// (x <- a x + b with the fixed point 1, so values stay normal); one output per thread
__global__ void __launch_bounds__(256) k_dfma_probe(double* __restrict__ out, int iters, double a, double b)
{
	double x[8];
#pragma unroll
	for (int i = 0; i < 8; ++i) x[i] = 1.0 + 1e-3 * (threadIdx.x + 37 * i);
	for (int it = 0; it < iters; ++it) {
#pragma unroll
		for (int i = 0; i < 8; ++i) x[i] = fma(x[i], a, b);
	}
	double s = 0.0;
#pragma unroll
	for (int i = 0; i < 8; ++i) s += x[i];
	out[(long)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int qpc_fp64_peak(double* tflops)
{
	if (!tflops) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	*tflops = 0.0;
	int dev = 0;
	if (int rc = check_device(&dev)) return rc;
	int nsm = 0;
	QPC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
	const int threads = 256, blocks = 4 * nsm, iters = 8192;
	double* out = nullptr;
	if (int rc = dalloc(&out, (size_t)blocks * threads)) return rc;	// one value per launched thread
	cudaStream_t st = nullptr;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	int rc = QPC_OK;
	if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
		cudaEventCreate(&e1) != cudaSuccess) { set_error("stream or event creation failed"); rc = QPC_ERR_CUDA; }
	float best = 0.f;
	for (int rep = 0; rep < 6 && !rc; ++rep) {	// the first launch warms up
		cudaEventRecord(e0, st);
		k_dfma_probe<<<blocks, threads, 0, st>>>(out, iters, 0.9999999, 1e-7);
		cudaEventRecord(e1, st);
		if (cudaGetLastError() != cudaSuccess) { set_error("probe launch failed"); rc = QPC_ERR_CUDA; break; }
		if ((rc = wait_on(st))) break;
		float ms = 0.f;
		cudaEventElapsedTime(&ms, e0, e1);
		if (rep > 0 && (best == 0.f || ms < best)) best = ms;
	}
	if (!rc && best > 0.f) *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
	if (!rc) { cudaFree(out); out = nullptr; }	// after a timeout the probe may still be running: keep its buffer
	if (e0) cudaEventDestroy(e0);
	if (e1) cudaEventDestroy(e1);
	if (st) cudaStreamDestroy(st);
	return rc;
}

int qpc_set_wait_limit(double seconds)
{
	if (!(seconds > 0) || !std::isfinite(seconds)) { set_error("wait limit %g s: must be positive and finite", seconds); return QPC_ERR_ARGS; }
	g_wait_limit.store(seconds, std::memory_order_relaxed);
	return QPC_OK;
}

double qpc_get_wait_limit(void) { return wait_limit_s(); }
const char* qpc_version(void) { return "qpc-gb300 engine 1 (sm_103a, complex FP64)"; }

static int create_impl(const qpc_dims* dims, double dt, const double* S, const double* R, const double* H, int hpi, qpc_lgwz** out)
{
	if (!out) { set_error("out is NULL"); return QPC_ERR_ARGS; }
	*out = nullptr;
	if (!dims || !S || !R || !H) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	const qpc_dims d = *dims;
	if (d.p < 3 || d.p > QPC_MAX_RANK || d.n_r < 2 * d.p + 2 || d.n_l < 1 || d.n_m < 1 || d.n_inst < 1 || !(dt > 0) || !std::isfinite(dt)) {
		set_error("bad dims n_r=%d p=%d n_l=%d n_m=%d n_inst=%d dt=%g", d.n_r, d.p, d.n_l, d.n_m, d.n_inst, dt);
		return QPC_ERR_ARGS;
	}
	int dev = 0;
	if (int rc = check_device(&dev)) return rc;
	auto* h = new (std::nothrow) qpc_lgwz();
	if (!h) { set_error("host allocation"); return QPC_ERR_NOMEM; }
	h->dev = dev; h->d = d; h->N = d.n_r; h->P = d.p; h->L = d.n_l; h->M = d.n_m; h->B = d.n_inst; h->dt = dt; h->hpi = hpi ? 1 : 0;
	long mabs = std::max(std::labs((long)d.m0), std::labs((long)d.m0 + d.n_m - 1));
	h->lmax = (int)(mabs + d.n_l - 1);
	h->nlh = h->lmax + 1;
	h->npair = d.n_l / 2;
	const int N = h->N, P = h->P, NE = P + 1, L = h->L, M = h->M, np = h->npair;
	int rc = QPC_OK;
	auto fail = [&](int code) { qpc_lgwz_destroy(h); return code; };
	if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) { set_error("stream create"); return fail(QPC_ERR_CUDA); }
	cudaEventCreate(&h->ev0); cudaEventCreate(&h->ev1); cudaEventCreate(&h->evt0); cudaEventCreate(&h->evt1);
	h->NS = d.n_inst >= 2 ? 2 : 1;
	if (const char* e = getenv("QPC_STREAMS")) h->NS = std::max(1, std::min(qpc_lgwz::MAXNS, std::min(d.n_inst, atoi(e))));
	for (int g = 0; g < h->NS; ++g) {
		if (cudaStreamCreateWithFlags(&h->gs[g], cudaStreamNonBlocking) != cudaSuccess) { set_error("stream create"); return fail(QPC_ERR_CUDA); }
		cudaEventCreateWithFlags(&h->gev[g], cudaEventDisableTiming);
	}
	cudaEventCreateWithFlags(&h->xev, cudaEventDisableTiming);
	// host setup: field-free LDL^T per l (per instance and l with hpi), Y10 eigensystems
	const int nff = h->hpi ? h->B : 1;
	std::vector<double2> ffh((size_t)N * NE * h->nlh * nff);
	std::vector<double> Lrow((size_t)N * P * 2), Dinv((size_t)N * 2);
	for (int fi = 0; fi < nff; ++fi)
		for (int l = 0; l < h->nlh; ++l) {
			const size_t bl = (size_t)fi * h->nlh + l;
			int bad = qpc_ldlt_csym(N, P, S, H + bl * N * NE, dt * 0.5, Lrow.data(), Dinv.data());
			if (bad < 0) { set_error("ldlt arguments"); return fail(QPC_ERR_ARGS); }
			if (bad > 0) { set_error("zero pivot factorising S + i dt/2 H_%d (instance %d)", l, fi); return fail(QPC_ERR_SINGULAR); }
			// row form per l: ff[l][r][c] = L(r, r-1-c), ff[l][r][P] = 1/D(r)
			for (int r = 0; r < N; ++r) {
				for (int c = 0; c < P; ++c)
					ffh[(bl * N + r) * NE + c] = make_double2(Lrow[2 * ((size_t)r * P + c)], Lrow[2 * ((size_t)r * P + c) + 1]);
				ffh[(bl * N + r) * NE + P] = make_double2(Dinv[2 * (size_t)r], Dinv[2 * (size_t)r + 1]);
			}
		}
	h->h_lam.assign((size_t)M * L, 0.0);
	h->h_P.assign((size_t)M * L * L, 0.0);
	std::vector<double> Vh((size_t)M * (np + 1) * L, 0.0), lamp((size_t)M * std::max(np, 1), 0.0);
	for (int im = 0; im < M; ++im) {
		double* lam = h->h_lam.data() + (size_t)im * L;
		double* Pm = h->h_P.data() + (size_t)im * L * L;
		if ((rc = qpc_y10_eigen(L, d.m0 + im, lam, Pm))) return fail(rc);
		for (int k = 0; k < np; ++k) {
			int row = L - 1 - k;	// +s_k
			lamp[(size_t)im * np + k] = lam[row];
			for (int il = 0; il < L; ++il) Vh[((size_t)im * (np + 1) + k) * L + il] = Pm[(size_t)row * L + il];
		}
		if (L & 1)
			for (int il = 0; il < L; ++il) Vh[((size_t)im * (np + 1) + np) * L + il] = Pm[(size_t)np * L + il];
	}
	// look-ahead depth of the coupling factorisation: ~40k independent systems per
	// launch (fills every FP64 pipe even for one wavefunction), in at most
	// min(4 GB, max(256 MB, 64 MB per wavefunction)) of factors, so that many small
	// handles can share one GPU; QPC_FAC_BYTES overrides the bound
	size_t per_step = (size_t)h->B * M * N * NE * std::max(np, 1) * sizeof(double2);
	size_t fac_cap = std::min<size_t>((size_t)4 << 30, std::max<size_t>((size_t)256 << 20, (size_t)h->B * (64 << 20)));
	if (const char* e = getenv("QPC_FAC_BYTES")) fac_cap = std::max<size_t>(per_step, (size_t)atoll(e));
	h->K = 1;
	while (h->K < 4096 && (long)h->K * h->B * M * np < 40000 && per_step * (h->K * 2) <= fac_cap) h->K *= 2;
	long sl = state_len(h);
	if ((rc = dalloc(&h->S, (size_t)N * NE)) || (rc = dalloc(&h->R, (size_t)N * NE)) || (rc = dalloc(&h->Vh, Vh.size())) ||
		(rc = dalloc(&h->lamp, lamp.size())) || (rc = dalloc(&h->ff, ffh.size())) || (rc = dalloc(&h->st, sl)) ||
		(rc = dalloc(&h->eo, sl)) || (rc = dalloc(&h->wk, sl)) ||
		(rc = dalloc(&h->hostlay, sl)) || (rc = dalloc(&h->fac, per_step / sizeof(double2) * h->K)) ||
		(rc = dalloc(&h->status, 1)) || (rc = dalloc(&h->red, (size_t)h->B * M * L * 2)) ||
		(rc = dalloc(&h->ntf, h->B)) || (rc = dalloc(&h->ntt, h->B)))
		return fail(rc);
	if (cudaMemcpy(h->S, S, sizeof(double) * N * NE, cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemcpy(h->R, R, sizeof(double) * N * NE, cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemcpy(h->Vh, Vh.data(), sizeof(double) * Vh.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemcpy(h->lamp, lamp.data(), sizeof(double) * lamp.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemcpy(h->ff, ffh.data(), sizeof(double2) * ffh.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemset(h->st, 0, sizeof(double2) * sl) != cudaSuccess || cudaMemset(h->status, 0, sizeof(int)) != cudaSuccess) {
		set_error("initial device copies failed");
		return fail(QPC_ERR_CUDA);
	}
	// segmented chain solver for few wavefunctions: Q <= 16 segments of Ls >= P rows, the last one >= P rows
	h->seg_ok = h->B <= 8 && np > 0;
	if (h->seg_ok) {
		auto fits = [&](int q) { const int ls = (N + q - 1) / q; return ls >= P && N - (q - 1) * ls >= P; };
		int q = 16;
		while (q > 1 && !fits(q)) --q;
		h->seg_ok = q >= 2;
		h->Q = q;
		h->Ls = (N + q - 1) / q;
		// stage the factor block in shared memory when it fits beside the kernel's static arrays
		int optin = 0;
		cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
		const long budget = (long)optin - 8 * 1024;
		for (int cpl = 0; cpl < 2; ++cpl) {
			const int nc = cpl ? 2 : 1;
			const long with = (long)sizeof(double2) * seg_smem_elems(N, P, nc, q, true);
			const long without = (long)sizeof(double2) * seg_smem_elems(N, P, nc, q, false);
			h->seg_sfac[cpl] = with <= budget;
			h->seg_smem[cpl] = (size_t)(h->seg_sfac[cpl] ? with : without);
			if (!h->seg_sfac[cpl] && without > budget) h->seg_ok = false;
		}
	}
	if (h->seg_ok) {
		const size_t nblk_ff = (size_t)nff * h->nlh, nblk_c = (size_t)h->K * h->B * M * np;
		std::vector<double2> sf(nblk_ff * N * P), sb(nblk_ff * N * P);
		switch (P) {
		case 3: host_spikes<3>(ffh.data(), nblk_ff, N, h->Q, h->Ls, sf.data(), sb.data()); break;
		case 4: host_spikes<4>(ffh.data(), nblk_ff, N, h->Q, h->Ls, sf.data(), sb.data()); break;
		case 5: host_spikes<5>(ffh.data(), nblk_ff, N, h->Q, h->Ls, sf.data(), sb.data()); break;
		case 6: host_spikes<6>(ffh.data(), nblk_ff, N, h->Q, h->Ls, sf.data(), sb.data()); break;
		case 7: host_spikes<7>(ffh.data(), nblk_ff, N, h->Q, h->Ls, sf.data(), sb.data()); break;
		case 8: host_spikes<8>(ffh.data(), nblk_ff, N, h->Q, h->Ls, sf.data(), sb.data()); break;
		}
		if ((rc = dalloc(&h->spf_ff, sf.size())) || (rc = dalloc(&h->spb_ff, sb.size())) ||
			(rc = dalloc(&h->spf_c, nblk_c * N * P)) || (rc = dalloc(&h->spb_c, nblk_c * N * P)))
			return fail(rc);
		if (cudaMemcpy(h->spf_ff, sf.data(), sizeof(double2) * sf.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
			cudaMemcpy(h->spb_ff, sb.data(), sizeof(double2) * sb.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
			cudaMemset(h->spf_c, 0, sizeof(double2) * nblk_c * N * P) != cudaSuccess ||
			cudaMemset(h->spb_c, 0, sizeof(double2) * nblk_c * N * P) != cudaSuccess) {
			set_error("initial device copies failed");
			return fail(QPC_ERR_CUDA);
		}
	}
	if (h->hpi) {
		std::vector<int> id(h->B);
		for (int k = 0; k < h->B; ++k) id[k] = k;
		if ((rc = dalloc(&h->ffmap, h->B)) || (rc = dalloc(&h->ffmap_id, h->B))) return fail(rc);
		if (cudaMemcpy(h->ffmap_id, id.data(), sizeof(int) * h->B, cudaMemcpyHostToDevice) != cudaSuccess) {
			set_error("initial device copies failed");
			return fail(QPC_ERR_CUDA);
		}
		h->ffmap_cur = h->ffmap_id;
	}
	const char* ltc = getenv("QPC_LTRANS_TC");
	h->lt_kb = (ltc && atoi(ltc) == 0) ? 0 : ltrans_kb(L);
	if (h->lt_kb && !(ltc && atoi(ltc) == 1)) {
		int nsm = 0;
		if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) nsm = 152;
		h->lt_min_tiles = nsm;
	}
	if (h->lt_kb) {
		std::vector<uint16_t> dig(ltrans_digit_bytes(M, h->lt_kb) / 2);
		std::vector<int> fex((size_t)M * 2 * 2 * h->lt_kb);
		ltrans_digits(Vh.data(), M, L, np, h->lt_kb, dig.data(), fex.data());
		if ((rc = dalloc(&h->lt_dig, dig.size())) || (rc = dalloc(&h->lt_fex, fex.size()))) return fail(rc);
		if (cudaMemcpy(h->lt_dig, dig.data(), sizeof(uint16_t) * dig.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
			cudaMemcpy(h->lt_fex, fex.data(), sizeof(int) * fex.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
			set_error("initial device copies failed");
			return fail(QPC_ERR_CUDA);
		}
	}
	size_t smem = sizeof(double2) * 2 * TR * (L | 1);
	h->chain_smem = sizeof(double) * (size_t)N * NE;
	if (const char* e = getenv("QPC_CHAIN_SSTAGE")) h->chain_sstage = atoi(e) ? 1 : 0;
	if (const char* e = getenv("QPC_CHAIN_WARPS")) h->chain_warps = std::max(1, std::min(CHAIN_MAXW, atoi(e)));
	if (h->chain_sstage && h->chain_smem > 200 * 1024) { set_error("n_r=%d too large for the shared-memory S band", N); return fail(QPC_ERR_ARGS); }
	set_smem_attrs(h, smem);
	std::memset(h->gsel, 0, sizeof(h->gsel));
	for (int g = 1; g <= P; ++g) if (P % g == 0 && (g <= 4 || g == P)) h->gcand.push_back(g);
	if (h->seg_ok) h->gcand.push_back(QPC_SEG);	// the segmented solver
	*out = h;
	return QPC_OK;
}

int qpc_lgwz_create(const qpc_dims* dims, double dt, const double* S, const double* R, const double* H, qpc_lgwz** out)
{
	return create_impl(dims, dt, S, R, H, 0, out);
}

int qpc_lgwz_create_ex(const qpc_dims* dims, double dt, const double* S, const double* R, const double* H, int32_t h_per_instance,
	qpc_lgwz** out)
{
	return create_impl(dims, dt, S, R, H, h_per_instance, out);
}

int qpc_lgwz_destroy(qpc_lgwz* h)
{
	if (!h) return QPC_OK;
	if (h->stream) cudaStreamSynchronize(h->stream);
	cudaFree(h->S); cudaFree(h->R); cudaFree(h->Vh); cudaFree(h->lamp); cudaFree(h->ff); cudaFree(h->lt_dig); cudaFree(h->lt_fex);
	cudaFree(h->ffmap); cudaFree(h->ffmap_id);
	cudaFree(h->spf_c); cudaFree(h->spb_c); cudaFree(h->spf_ff); cudaFree(h->spb_ff);
	cudaFree(h->st); cudaFree(h->eo); cudaFree(h->wk); cudaFree(h->hostlay); cudaFree(h->fac);
	cudaFree(h->status); cudaFree(h->red); cudaFree(h->ntf); cudaFree(h->ntt); cudaFree(h->ftab);
	cudaFree(h->obsF); cudaFree(h->obs); cudaFree(h->dl); cudaFree(h->y10d); cudaFree(h->zdev);
	cudaFree(h->mM); cudaFree(h->mLrow); cudaFree(h->mLcol); cudaFree(h->mdinv); cudaFree(h->slotmap);
	for (auto e : h->evpool) cudaEventDestroy(e);
	for (int g = 0; g < qpc_lgwz::MAXNS; ++g) {
		if (h->gs[g]) { cudaStreamSynchronize(h->gs[g]); cudaStreamDestroy(h->gs[g]); }
		if (h->gev[g]) cudaEventDestroy(h->gev[g]);
		if (g == 0 && h->xev) cudaEventDestroy(h->xev);
	}
	if (h->evt0) cudaEventDestroy(h->evt0);
	if (h->evt1) cudaEventDestroy(h->evt1);
	if (h->ev0) cudaEventDestroy(h->ev0);
	if (h->ev1) cudaEventDestroy(h->ev1);
	if (h->stream) cudaStreamDestroy(h->stream);
	delete h;
	return QPC_OK;
}

static int put_common(qpc_lgwz* h, const double* src, cudaMemcpyKind kind)
{
	long sl = state_len(h);
	// the stream idle first: a copy from pageable memory then never waits for queued work
	if (kind == cudaMemcpyHostToDevice) if (int rc = wait_stream(h)) return rc;
	QPC_CUDA(cudaMemcpyAsync(h->hostlay, src, sizeof(double2) * sl, kind, h->stream));
	long nblk = (long)h->B * h->M;
	k_to_rmajor<<<(unsigned)((sl + 255) / 256), 256, 0, h->stream>>>(h->hostlay, h->st, h->N, h->L, nblk);
	LAUNCH(h);
	QPC_CUDA(cudaGetLastError());
	return wait_stream(h);
}
static int get_common(qpc_lgwz* h, double* dst, cudaMemcpyKind kind)
{
	long sl = state_len(h);
	long nblk = (long)h->B * h->M;
	k_to_lmajor<<<(unsigned)((sl + 255) / 256), 256, 0, h->stream>>>(h->st, h->hostlay, h->N, h->L, nblk);
	LAUNCH(h);
	QPC_CUDA(cudaGetLastError());
	if (kind == cudaMemcpyDeviceToHost) return copy_to_host(dst, h->hostlay, sizeof(double2) * sl, h->stream);
	QPC_CUDA(cudaMemcpyAsync(dst, h->hostlay, sizeof(double2) * sl, kind, h->stream));
	return wait_stream(h);
}

int qpc_lgwz_put(qpc_lgwz* h, const double* coef)
{
	if (!h || !coef) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	return put_common(h, coef, cudaMemcpyHostToDevice);
}
int qpc_lgwz_get(qpc_lgwz* h, double* coef)
{
	if (!h || !coef) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	return get_common(h, coef, cudaMemcpyDeviceToHost);
}
int qpc_lgwz_put_device(qpc_lgwz* h, const double* dev_coef)
{
	if (!h || !dev_coef) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	return put_common(h, dev_coef, cudaMemcpyDeviceToDevice);
}
int qpc_lgwz_get_device(qpc_lgwz* h, double* dev_coef)
{
	if (!h || !dev_coef) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	return get_common(h, dev_coef, cudaMemcpyDeviceToDevice);
}
int qpc_lgwz_dims(qpc_lgwz* h, qpc_dims* dims)
{
	if (!h || !dims) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	*dims = h->d;
	return QPC_OK;
}
int qpc_lgwz_stream(qpc_lgwz* h, void** stream)
{
	if (!h || !stream) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	*stream = (void*)h->stream;
	return QPC_OK;
}

static int mask_prepare(qpc_lgwz* h);
static void mask_enqueue(qpc_lgwz* h, cudaStream_t st, const int64_t* ntt, long step);

static int run_impl(qpc_lgwz* h, const double* ftab, int64_t ld, const int64_t* nt_field, const int64_t* nt_total,
	const double* F, double* zlist, int64_t ldz, const qpc_run_opts* opts = nullptr)
{
	if (!h || !nt_field || !nt_total) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	QPC_CUDA(cudaSetDevice(h->dev));
	// the stream idle first (bounded): the copies from host memory below then never wait
	// for queued work (after a call that timed out, the work it left is waited for here)
	if (int rc = wait_stream(h)) return rc;
	h->observing = false;
	const int B = h->B;
	long smax = 0;
	bool anyfield = false;
	for (int k = 0; k < B; ++k) {
		if (nt_field[k] < 0 || nt_total[k] < nt_field[k]) { set_error("instance %d: nt_field=%lld nt_total=%lld", k, (long long)nt_field[k], (long long)nt_total[k]); return QPC_ERR_ARGS; }
		if (nt_field[k] > 0) { anyfield = true; if (ld < nt_field[k] + 1) { set_error("ld=%lld < nt_field+1", (long long)ld); return QPC_ERR_ARGS; } }
		smax = std::max<long>(smax, std::max<long>(nt_total[k], nt_field[k] + (nt_field[k] > 0 ? 1 : 0)));
	}
	if (anyfield && !ftab) { set_error("ftab is NULL"); return QPC_ERR_ARGS; }
	const double* mband = opts ? opts->mask : nullptr;
	qpc_tsurff* tsf = opts ? opts->tsurff : nullptr;
	const bool split = mband || tsf;
	if (split && F) { set_error("the in-loop dipole and the per-step mask or t-SURFF cannot be combined in one run"); return QPC_ERR_ARGS; }
	if (tsf) if (int rc = tsurff_check_grid(tsf, h->d)) return rc;
	long ntt_max = 0;
	for (int k = 0; k < B; ++k) ntt_max = std::max<long>(ntt_max, nt_total[k]);
	// field table to the device, padded to B*ld
	size_t need = anyfield ? (size_t)B * ld : 1;
	if (h->ftab_cap < need) {
		cudaFree(h->ftab); h->ftab = nullptr; h->ftab_cap = 0;
		if (int rc = dalloc(&h->ftab, need)) return rc;
		h->ftab_cap = need;
	}
	if (anyfield) {
		for (int k = 0; k < B; ++k)
			for (int64_t i = 0; i <= nt_field[k]; ++i)
				if (nt_field[k] > 0 && !std::isfinite(ftab[(size_t)k * ld + i])) { set_error("non-finite field value, instance %d step %lld", k, (long long)i); return QPC_ERR_ARGS; }
		QPC_CUDA(cudaMemcpyAsync(h->ftab, ftab, sizeof(double) * need, cudaMemcpyHostToDevice, h->stream));
	}
	// Instances are processed in decreasing order of nt_field (then nt_total):
	// the instances still in their pulse at step s are then a prefix, and
	// launches cover only that prefix.
	std::vector<int> perm(B);
	std::iota(perm.begin(), perm.end(), 0);
	std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) {
		return nt_field[x] != nt_field[y] ? nt_field[x] > nt_field[y] : nt_total[x] > nt_total[y]; });
	bool ident = true;
	for (int k = 0; k < B; ++k) ident &= perm[k] == k;
	std::vector<int64_t> pf(B), pt(B);
	for (int k = 0; k < B; ++k) { pf[k] = nt_field[perm[k]]; pt[k] = nt_total[perm[k]]; }
	if (anyfield && !ident) {
		std::vector<double> tab((size_t)B * ld);
		for (int k = 0; k < B; ++k) std::memcpy(tab.data() + (size_t)k * ld, ftab + (size_t)perm[k] * ld, sizeof(double) * ld);
		QPC_CUDA(cudaMemcpyAsync(h->ftab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, h->stream));
		if (int rc = wait_stream(h)) return rc;
	}
	QPC_CUDA(cudaMemcpyAsync(h->ntf, pf.data(), sizeof(int64_t) * B, cudaMemcpyHostToDevice, h->stream));
	QPC_CUDA(cudaMemcpyAsync(h->ntt, pt.data(), sizeof(int64_t) * B, cudaMemcpyHostToDevice, h->stream));
	// own potentials: the sorted instance k uses the field-free factors of instance perm[k]
	struct map_restore { qpc_lgwz* h; ~map_restore() { if (h->hpi) h->ffmap_cur = h->ffmap_id; } } mr{h};
	if (h->hpi) {
		QPC_CUDA(cudaMemcpyAsync(h->ffmap, perm.data(), sizeof(int) * B, cudaMemcpyHostToDevice, h->stream));
		h->ffmap_cur = h->ffmap;
	}
	QPC_CUDA(cudaMemsetAsync(h->status, 0, sizeof(int), h->stream));
	if (!ident) if (int rc = permute_instances(h, perm, false)) return rc;
	h->ld = anyfield ? (long)ld : 0;
	if (F) {
		const int N = h->N, NE = h->P + 1, M = h->M, L = h->L;
		long ntmax = 0;
		for (int k = 0; k < B; ++k) ntmax = std::max<long>(ntmax, nt_total[k]);
		if (!zlist || ldz < ntmax) { set_error("zlist NULL or ldz=%lld < max nt_total=%ld", (long long)ldz, ntmax); return QPC_ERR_ARGS; }
		if (!h->obsF) {
			std::vector<double> y((size_t)M * L);
			for (int m = 0; m < M; ++m) qpc_y10_coupling(L, h->d.m0 + m, y.data() + (size_t)m * L);
			int rc;
			if ((rc = dalloc(&h->obsF, (size_t)N * NE)) || (rc = dalloc(&h->obs, (size_t)B * M * std::max(h->npair, 1) * 2)) ||
				(rc = dalloc(&h->dl, (size_t)B * M * L)) || (rc = dalloc(&h->y10d, (size_t)M * L)))
				return rc;
			QPC_CUDA(cudaMemcpyAsync(h->y10d, y.data(), sizeof(double) * y.size(), cudaMemcpyHostToDevice, h->stream));
			if (int rc2 = wait_stream(h)) return rc2;
		}
		if (h->zcap < (size_t)B * ldz) {
			cudaFree(h->zdev); h->zdev = nullptr; h->zcap = 0;
			if (int rc = dalloc(&h->zdev, (size_t)B * ldz)) return rc;
			h->zcap = (size_t)B * ldz;
		}
		QPC_CUDA(cudaMemcpyAsync(h->obsF, F, sizeof(double) * N * NE, cudaMemcpyHostToDevice, h->stream));
		QPC_CUDA(cudaMemsetAsync(h->zdev, 0, sizeof(double) * B * ldz, h->stream));
		if (int rc = wait_stream(h)) return rc;
		h->ldz = ldz;
		h->observing = true;
	}
	// Instance groups (contiguous in the sorted order, balanced by work) on their
	// own streams; within a group, the instances still in their pulse at step s
	// are a prefix, and the field-free ones lie below a bound.
	const int NS = h->NS;
	std::vector<int> gb(NS + 1, 0);
	{
		double tot = 0.0;
		for (int k = 0; k < B; ++k) tot += (double)pt[k] + 2.0 * pf[k];
		double acc = 0.0;
		int g = 1;
		for (int k = 0; k < B && g < NS; ++k) {
			acc += (double)pt[k] + 2.0 * pf[k];
			if (acc >= tot * g / NS) gb[g++] = k + 1;
		}
		for (; g < NS; ++g) gb[g] = B;
		gb[NS] = B;
		for (int q = 1; q <= NS; ++q) gb[q] = std::max(gb[q], gb[q - 1]);
	}
	std::vector<int> Bc(NS), Bf(NS);
	auto live_counts = [&](long s) {
		for (int g = 0; g < NS; ++g) {
			int n = 0;
			while (gb[g] + n < gb[g + 1] && pf[gb[g] + n] > 0 && pf[gb[g] + n] >= s) ++n;
			int f = gb[g + 1] - gb[g];
			while (f > 0 && pt[gb[g] + f - 1] <= s) --f;
			Bc[g] = n; Bf[g] = f;
		}
	};
	// per-step extras: the mask band and the slot map the t-SURFF prepare reads
	std::vector<double> ta((size_t)2 * B);
	std::vector<int> tact(B);
	between_steps extras;
	if (split) {
		if (mband) {
			if (int rc = mask_prepare(h)) return rc;
			QPC_CUDA(cudaMemcpyAsync(h->mM, mband, sizeof(double) * h->N * (h->P + 1), cudaMemcpyHostToDevice, h->stream));
		}
		if (tsf) {
			if (!h->slotmap) if (int rc = dalloc(&h->slotmap, (size_t)B)) return rc;
			std::vector<int> slot(B);
			for (int k = 0; k < B; ++k) slot[perm[k]] = k;
			QPC_CUDA(cudaMemcpyAsync(h->slotmap, slot.data(), sizeof(int) * B, cudaMemcpyHostToDevice, h->stream));
		}
		if (int rc = wait_stream(h)) return rc;
		// after step s - 1 of instance i (1 <= s <= nt_total[i]): accumulate with (f(t_s-1), f(t_s))
		// while in the pulse, the field-free accumulate (zero field) after it, then the mask
		extras.fn = [&](long s) -> int {
			bool any = false;
			for (int i = 0; i < B; ++i) {
				tact[i] = (s >= 1 && s <= nt_total[i]) ? 1 : 0;
				any |= tact[i] != 0;
				const bool fld = s - 1 < nt_field[i];
				ta[2 * (size_t)i] = fld ? ftab[(size_t)i * ld + s - 1] : 0.0;
				ta[2 * (size_t)i + 1] = fld ? ftab[(size_t)i * ld + s] : 0.0;
			}
			if (!any) return QPC_OK;
			if (tsf) if (int rc = tsurff_enqueue_engine(tsf, h->st, h->slotmap, ta.data(), tact.data(), h->dt, (void*)h->stream)) return rc;
			if (mband) mask_enqueue(h, h->stream, h->ntt, s);
			return QPC_OK;
		};
	}
	// with extras every coupling step is split and the loop runs one more step (the extras after the last step)
	const long send = split ? ntt_max + 1 : smax;
	QPC_CUDA(cudaEventRecord(h->ev0, h->stream));
	for (int g = 0; g < NS; ++g) QPC_CUDA(cudaStreamWaitEvent(h->gs[g], h->ev0, 0));
	for (long s = 0; s < send; ++s) {
		// factors for steps s .. s+K-1 are computed together, into slots 0..K-1
		int j = (int)(s % h->K);
		long kf = std::min<long>(h->K, send - s);
		live_counts(s);
		if (split) {
			if (int rc = launch_split(h, s, s - j, j, j == 0, (int)kf, gb.data(), Bc.data(), Bf.data(), extras)) return rc;
		} else if (int rc = launch_step(h, s, s - j, j, j == 0, (int)kf, gb.data(), Bc.data(), Bf.data())) return rc;
	}
	for (int g = 0; g < NS; ++g) {
		QPC_CUDA(cudaEventRecord(h->gev[g], h->gs[g]));
		QPC_CUDA(cudaStreamWaitEvent(h->stream, h->gev[g], 0));
	}
	QPC_CUDA(cudaEventRecord(h->ev1, h->stream));
	QPC_CUDA(cudaGetLastError());
	h->observing = false;
	if (!ident) if (int rc = permute_instances(h, perm, true)) return rc;
	long sl = state_len(h);
	k_status_check<<<(unsigned)((sl + 255) / 256), 256, 0, h->stream>>>(h->st, sl, h->status);
	LAUNCH(h);
	int rc = read_status(h);
	float ms = 0.f;
	cudaEventElapsedTime(&ms, h->ev0, h->ev1);
	h->last_ms = ms;
	collect_profile(h);
	if (F && rc == QPC_OK) {
		std::vector<double> zh((size_t)B * ldz);
		if (int rc2 = copy_to_host(zh.data(), h->zdev, sizeof(double) * zh.size(), h->stream)) return rc2;
		for (int k = 0; k < B; ++k) std::memcpy(zlist + (size_t)perm[k] * ldz, zh.data() + (size_t)k * ldz, sizeof(double) * ldz);
	}
	return rc;
}

int qpc_lgwz_run(qpc_lgwz* h, const double* ftab, int64_t ld, const int64_t* nt_field, const int64_t* nt_total)
{
	return run_impl(h, ftab, ld, nt_field, nt_total, nullptr, nullptr, 0);
}

int qpc_lgwz_run_ex(qpc_lgwz* h, const double* ftab, int64_t ld, const int64_t* nt_field, const int64_t* nt_total, const qpc_run_opts* opts)
{
	return run_impl(h, ftab, ld, nt_field, nt_total, nullptr, nullptr, 0, opts);
}

// Several handles at once: one host thread per handle, each driving its handle's
// own streams, so that batches on different grids share the GPU.
int qpc_lgwz_run_many(int32_t n, qpc_lgwz* const* hs, const double* const* ftab, const int64_t* ld,
	const int64_t* const* nt_field, const int64_t* const* nt_total, int32_t* failed)
{
	if (failed) *failed = -1;
	if (n < 0 || (n > 0 && (!hs || !ld || !nt_field || !nt_total))) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	for (int i = 0; i < n; ++i)
		for (int j = 0; j < i; ++j)
			if (hs[i] == hs[j]) { set_error("handle %d appears twice", i); return QPC_ERR_ARGS; }
	std::vector<int> rc(n, QPC_OK);
	std::vector<std::string> msg(n);
	std::vector<std::thread> th;
	th.reserve(n);
	for (int i = 0; i < n; ++i)
		th.emplace_back([&, i] {
			rc[i] = qpc_lgwz_run(hs[i], ftab ? ftab[i] : nullptr, ld[i], nt_field[i], nt_total[i]);
			if (rc[i]) msg[i] = qpc_last_error();
		});
	for (auto& t : th) t.join();
	for (int i = 0; i < n; ++i)
		if (rc[i]) {
			if (failed) *failed = i;
			set_error("handle %d: %s", i, msg[i].c_str());
			return rc[i];
		}
	return QPC_OK;
}

int qpc_lgwz_run_dipole(qpc_lgwz* h, const double* ftab, int64_t ld, const int64_t* nt_field, const int64_t* nt_total,
	const double* F, double* zlist, int64_t ldz)
{
	if (!F) { set_error("F is NULL"); return QPC_ERR_ARGS; }
	return run_impl(h, ftab, ld, nt_field, nt_total, F, zlist, ldz);
}

int qpc_lgwz_propagate(qpc_lgwz* h, const double* f_ti, const double* f_tf)
{
	if (!h || !f_ti || !f_tf) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	std::vector<double> tab((size_t)h->B * 2);
	std::vector<int64_t> nf(h->B, 1), nt(h->B, 1);
	for (int k = 0; k < h->B; ++k) { tab[2 * (size_t)k] = f_ti[k]; tab[2 * (size_t)k + 1] = f_tf[k]; }
	return qpc_lgwz_run(h, tab.data(), 2, nf.data(), nt.data());
}

int qpc_lgwz_propagate_free(qpc_lgwz* h)
{
	if (!h) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	std::vector<int64_t> nf(h->B, 0), nt(h->B, 1);
	return qpc_lgwz_run(h, nullptr, 1, nf.data(), nt.data());
}

int qpc_lgwz_norm(qpc_lgwz* h, double* norm)
{
	if (!h || !norm) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	long nch = (long)h->B * h->M * h->L;
	k_band_inner<<<(unsigned)((nch + 127) / 128), 128, 0, h->stream>>>(h->st, h->S, h->P + 1, h->N, h->L, nch, 0, h->red);
	LAUNCH(h);
	QPC_CUDA(cudaGetLastError());
	std::vector<double2> part(nch);
	if (int rc = copy_to_host(part.data(), h->red, sizeof(double2) * nch, h->stream)) return rc;
	long per = (long)h->M * h->L;
	for (int k = 0; k < h->B; ++k) {
		double s = 0.0;
		for (long c = 0; c < per; ++c) s += part[(size_t)k * per + c].x;
		norm[k] = s;
	}
	return QPC_OK;
}

// the Cholesky factor of S for the mask's S^-1, once per handle (absorber.hpp:51-63)
static int mask_prepare(qpc_lgwz* h)
{
	if (h->mLrow) return QPC_OK;
	const int N = h->N, P = h->P, NE = P + 1;
	std::vector<double> S((size_t)N * NE), Lc((size_t)N * NE);
	QPC_CUDA(cudaMemcpy(S.data(), h->S, sizeof(double) * S.size(), cudaMemcpyDeviceToHost));
	int bad = qpc_cholesky_band(N, P, S.data(), Lc.data());
	if (bad) { set_error("S is not positive definite (pivot %d)", bad); return QPC_ERR_SINGULAR; }
	std::vector<double> lrow((size_t)N * P, 0.0), lcol((size_t)N * P, 0.0), di(N);
	for (int r = 0; r < N; ++r) {
		di[r] = 1.0 / Lc[(size_t)r * NE];
		for (int j = 1; j <= P; ++j) {
			if (r - j >= 0) lrow[(size_t)r * P + j - 1] = Lc[(size_t)(r - j) * NE + j];
			if (r + j < N) lcol[(size_t)r * P + j - 1] = Lc[(size_t)r * NE + j];
		}
	}
	int rc;
	if ((rc = dalloc(&h->mM, (size_t)N * NE)) || (rc = dalloc(&h->mLrow, (size_t)N * P)) || (rc = dalloc(&h->mLcol, (size_t)N * P)) ||
		(rc = dalloc(&h->mdinv, (size_t)N)))
		return rc;
	QPC_CUDA(cudaMemcpy(h->mLrow, lrow.data(), sizeof(double) * lrow.size(), cudaMemcpyHostToDevice));
	QPC_CUDA(cudaMemcpy(h->mLcol, lcol.data(), sizeof(double) * lcol.size(), cudaMemcpyHostToDevice));
	QPC_CUDA(cudaMemcpy(h->mdinv, di.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
	return QPC_OK;
}

// c <- S^-1 (M c) on the resident state with the band in h->mM, enqueued on st; inside a run
// (ntt != NULL) only the instances whose step `step - 1` has just finished
static void mask_enqueue(qpc_lgwz* h, cudaStream_t st, const int64_t* ntt, long step)
{
	const int N = h->N, P = h->P;
	const long total = state_len(h);
	const long per = (long)h->M * N * h->L;
	k_mask_band<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(h->st, h->wk, h->mM, N, P, h->L, total, ntt, step, per);
	LAUNCH(h);
	const long nchain = 2L * h->B * h->M * h->L;
	const unsigned nb = (unsigned)((nchain + 63) / 64);
	switch (P) {
	case 1: k_mask_solve<1><<<nb, 64, 0, st>>>(h->st, h->wk, h->mLrow, h->mLcol, h->mdinv, N, h->L, nchain, ntt, step, h->M); break;
	case 2: k_mask_solve<2><<<nb, 64, 0, st>>>(h->st, h->wk, h->mLrow, h->mLcol, h->mdinv, N, h->L, nchain, ntt, step, h->M); break;
	case 3: k_mask_solve<3><<<nb, 64, 0, st>>>(h->st, h->wk, h->mLrow, h->mLcol, h->mdinv, N, h->L, nchain, ntt, step, h->M); break;
	case 4: k_mask_solve<4><<<nb, 64, 0, st>>>(h->st, h->wk, h->mLrow, h->mLcol, h->mdinv, N, h->L, nchain, ntt, step, h->M); break;
	case 5: k_mask_solve<5><<<nb, 64, 0, st>>>(h->st, h->wk, h->mLrow, h->mLcol, h->mdinv, N, h->L, nchain, ntt, step, h->M); break;
	case 6: k_mask_solve<6><<<nb, 64, 0, st>>>(h->st, h->wk, h->mLrow, h->mLcol, h->mdinv, N, h->L, nchain, ntt, step, h->M); break;
	case 7: k_mask_solve<7><<<nb, 64, 0, st>>>(h->st, h->wk, h->mLrow, h->mLcol, h->mdinv, N, h->L, nchain, ntt, step, h->M); break;
	default: k_mask_solve<8><<<nb, 64, 0, st>>>(h->st, h->wk, h->mLrow, h->mLcol, h->mdinv, N, h->L, nchain, ntt, step, h->M); break;
	}
	LAUNCH(h);
}

int qpc_lgwz_mask(qpc_lgwz* h, const double* M)
{
	if (!h || !M) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	const int N = h->N, NE = h->P + 1;
	if (int rc = wait_stream(h)) return rc;
	if (int rc = mask_prepare(h)) return rc;
	QPC_CUDA(cudaMemcpyAsync(h->mM, M, sizeof(double) * N * NE, cudaMemcpyHostToDevice, h->stream));
	mask_enqueue(h, h->stream, nullptr, 0);
	QPC_CUDA(cudaGetLastError());
	return wait_stream(h);
}

int qpc_lgwz_dipole(qpc_lgwz* h, const double* F, double* out)
{
	if (!h || !F || !out) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	const int N = h->N, NE = h->P + 1, L = h->L, M = h->M;
	if (int rc = wait_stream(h)) return rc;
	// stream-ordered scratch: freed in stream order, so no later wait can block on it
	double* dF = nullptr;
	if (cudaMallocAsync((void**)&dF, sizeof(double) * N * NE, h->stream) != cudaSuccess) { set_error("cudaMallocAsync failed"); return QPC_ERR_NOMEM; }
	long nch = (long)h->B * M * L;
	double2* red2 = h->red + nch;
	int rc = QPC_OK;
	if (cudaMemcpyAsync(dF, F, sizeof(double) * N * NE, cudaMemcpyHostToDevice, h->stream) != cudaSuccess) rc = QPC_ERR_CUDA;
	if (!rc) {
		k_band_inner<<<(unsigned)((nch + 127) / 128), 128, 0, h->stream>>>(h->st, dF, NE, N, L, nch, -1, h->red);
		k_band_inner<<<(unsigned)((nch + 127) / 128), 128, 0, h->stream>>>(h->st, dF, NE, N, L, nch, +1, red2);
		h->launches += 2;
		if (cudaGetLastError() != cudaSuccess) rc = QPC_ERR_CUDA;
	}
	cudaFreeAsync(dF, h->stream);
	if (rc) { set_error("dipole device step failed"); return rc; }
	std::vector<double2> lo(nch), hi(nch);
	if ((rc = copy_to_host(lo.data(), h->red, sizeof(double2) * nch, h->stream)) ||
		(rc = copy_to_host(hi.data(), red2, sizeof(double2) * nch, h->stream))) return rc;
	std::vector<double> y(L);
	for (int k = 0; k < h->B; ++k) {
		double re = 0.0, im = 0.0;
		for (int m = 0; m < M; ++m) {
			qpc_y10_coupling(L, h->d.m0 + m, y.data());
			for (int il = 0; il < L; ++il) {
				size_t c = ((size_t)k * M + m) * L + il;
				if (il > 0) { re += lo[c].x * y[il - 1]; im += lo[c].y * y[il - 1]; }
				if (il + 1 < L) { re += hi[c].x * y[il]; im += hi[c].y * y[il]; }
			}
		}
		out[2 * (size_t)k] = re; out[2 * (size_t)k + 1] = im;
	}
	return QPC_OK;
}

int qpc_lgwz_projection(qpc_lgwz* h, const int32_t* n_state, const double* basis, double* proj)
{
	if (!h || !n_state || !basis || !proj) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	const int N = h->N, L = h->L, M = h->M, nl = h->nlh;
	std::vector<long> boff(nl + 1, 0);
	int nmax = 0;
	for (int l = 0; l < nl; ++l) {
		if (n_state[l] < 0 || n_state[l] > N) { set_error("n_state[%d]=%d", l, n_state[l]); return QPC_ERR_ARGS; }
		boff[l + 1] = boff[l] + (long)n_state[l] * N;
		nmax = std::max(nmax, n_state[l]);
	}
	long nch = (long)h->B * M * L;
	std::vector<long> poff(nch + 1, 0);
	for (long c = 0; c < nch; ++c) {
		int il = (int)(c % L), m = (int)((c / L) % M) + h->d.m0;
		int l = il + (m < 0 ? -m : m);
		poff[c + 1] = poff[c] + n_state[l];
	}
	if (nmax == 0) return QPC_OK;
	if (int rc = wait_stream(h)) return rc;
	// stream-ordered scratch: freed in stream order, so no later wait can block on it
	void* buf[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
	const size_t bytes[5] = {sizeof(double) * (size_t)std::max<long>(boff[nl], 1), sizeof(long) * (nl + 1), sizeof(long) * (nch + 1),
		sizeof(int) * (size_t)nl, sizeof(double2) * (size_t)std::max<long>(poff[nch], 1)};
	bool ok = true;
	for (int i = 0; i < 5 && ok; ++i) ok = cudaMallocAsync(&buf[i], bytes[i], h->stream) == cudaSuccess;
	double* db = (double*)buf[0]; long* dbo = (long*)buf[1]; long* dpo = (long*)buf[2]; int* dn = (int*)buf[3]; double2* dp = (double2*)buf[4];
	ok = ok && cudaMemcpyAsync(db, basis, sizeof(double) * boff[nl], cudaMemcpyHostToDevice, h->stream) == cudaSuccess &&
		cudaMemcpyAsync(dbo, boff.data(), sizeof(long) * (nl + 1), cudaMemcpyHostToDevice, h->stream) == cudaSuccess &&
		cudaMemcpyAsync(dpo, poff.data(), sizeof(long) * (nch + 1), cudaMemcpyHostToDevice, h->stream) == cudaSuccess &&
		cudaMemcpyAsync(dn, n_state, sizeof(int) * nl, cudaMemcpyHostToDevice, h->stream) == cudaSuccess;
	if (ok) {
		long tot = nch * nmax;
		k_projection<<<(unsigned)((tot + 127) / 128), 128, 0, h->stream>>>(h->st, db, dbo, dn, dpo, N, L, M, h->d.m0, nch, nmax, dp);
		LAUNCH(h);
		ok = cudaGetLastError() == cudaSuccess;
	}
	int rc = ok ? copy_to_host(proj, dp, sizeof(double2) * poff[nch], h->stream) : QPC_ERR_CUDA;
	if (!ok) set_error("projection device step failed");
	for (int i = 0; i < 5; ++i) if (buf[i]) cudaFreeAsync(buf[i], h->stream);
	return rc;
}

int qpc_lgwz_last_run_ms(qpc_lgwz* h, double* ms)
{
	if (!h || !ms) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	*ms = h->last_ms;
	return QPC_OK;
}

int64_t qpc_lgwz_launch_count(qpc_lgwz* h) { return h ? h->launches : -1; }

int qpc_lgwz_set_profiling(qpc_lgwz* h, int on)
{
	if (!h) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	h->profiling = on != 0;
	for (int k = 0; k < QPC_NKERNEL; ++k) { h->kms[k] = 0.0; h->kcount[k] = 0; }
	return QPC_OK;
}

int qpc_lgwz_get_tuning(qpc_lgwz* h, int32_t* out)
{
	if (!h || !out) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	out[0] = h->K;
	for (int b = 0; b < 32; ++b) { out[1 + b] = h->gsel[1][b]; out[33 + b] = h->gsel[0][b]; }
	return QPC_OK;
}

int qpc_lgwz_kernel_times(qpc_lgwz* h, double* ms, int64_t* launches)
{
	if (!h || !ms || !launches) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	for (int k = 0; k < QPC_NKERNEL; ++k) { ms[k] = h->kms[k]; launches[k] = h->kcount[k]; }
	return QPC_OK;
}

} // extern "C"
