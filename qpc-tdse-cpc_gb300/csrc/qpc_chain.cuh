// Banded Crank-Nicolson chain solver for GB300.
//
// Every channel ("chain") of the propagation applies, a = 1 or 2 times,
//     z <- (S + i a B)^-1 (S - i a B) z = 2 (S + i a B)^-1 (S z) - z
// with the complex-symmetric band factorised as L D L^T (unit lower L with p
// sub-diagonals, stored row-wise: Lrow[r][k-1] = L(r, r-k), and 1/D(r)).
// This is the solve of cn_propagate_kernel_avx1 (coupling, propagate.hpp:3-98)
// and of cn_hc_propagate0 (field-free, propagate.hpp:311-331) rewritten as
//     P1  w = S z                       (rows independent)
//     P2  y = L^-1 w                    (recurrence over r, ascending)
//     P3  y <- D^-1 y                   (rows independent)
//     P4  x = L^-T y                    (recurrence over r, descending)
//     P5  z <- 2 x - z                  (rows independent)
// GB300 issues one FP64 warp instruction per ~64 cycles per SM sub-partition,
// whether the instruction depends on the previous one or not, so a recurrence
// advances one row per (FP64 instructions per lane per row) x 64 cycles.  The
// recurrences P2/P4 are therefore run column-oriented on a systolic window:
// G lanes per real/imaginary part each keep P/G of the P pending partial sums;
// when row c completes, its value is broadcast and every lane subtracts its
// L(c+j, c) * y_c in 2 P/G FMAs, then the window slides by one row
// (shuffles, no FP64).  The row-parallel passes P1/P3/P5 use all 32 lanes.
// One warp owns CPW chains and runs all passes itself (__syncwarp between),
// so no block-level synchronisation is needed.  G is chosen per batch size
// by the engine's autotuner: G = P gives the shortest rows (few chains,
// latency-bound), G = 1 the fewest idle lanes (many chains).
#pragma once

// prefetch distances for 1 and 2 partial sums per lane (compile-time tuning)
#ifndef QPC_CHAIN_PD1
#define QPC_CHAIN_PD1 16
#endif
#ifndef QPC_CHAIN_PD2
#define QPC_CHAIN_PD2 3
#endif

namespace qpc {

// Coupling chains come in pairs (+s, -s) that share one factorisation; the
// -s chain holds conj(z) and is solved with the +s factors.
template <int P, int G, bool CPL>
struct chain_cfg {
	static constexpr int NE = P + 1;
	static constexpr int LPC = 2 * G;	// lanes per chain: G real-part lanes, G imaginary-part lanes
	static constexpr int CPW = CPL ? ((32 / LPC) & ~1) : (32 / LPC);
	static constexpr int TPL = P / G;	// partial sums per lane
	// prefetch distance (columns) of the recurrences: a row costs 2*TPL FP64
	// instructions (~128*TPL cycles); memory latency is ~600-800 cycles
	static constexpr int PD = TPL >= 6 ? 1 : (TPL >= 3 ? 2 : (TPL == 2 ? QPC_CHAIN_PD2 : QPC_CHAIN_PD1));
	static_assert(P % G == 0, "G must divide P");
	static_assert(CPW >= 1, "too many lanes per chain");
};

// coupling applications of an instance with nt field steps at loop step s.  cmode 0 (fused): the
// closing half of step s-1 and the opening half of step s together (M^2 with one factorisation);
// cmode 1: the closing half only; cmode 2: the opening half only (a run that acts on the state
// between two steps, e.g. with an absorbing mask, splits every coupling step in two)
__device__ __forceinline__ int coupling_power(long s, long nt, int cmode = 0)
{
	if (nt <= 0) return 0;
	if (cmode == 1) return (s >= 1 && s <= nt) ? 1 : 0;
	if (cmode == 2) return s < nt ? 1 : 0;
	if (s > nt) return 0;
	return (s == 0 || s == nt) ? 1 : 2;
}

struct chain_desc {
	long xoff;	// offset of the chain's element at row 0 (double2 units); row stride = L
	long foff;	// offset of the chain's factor block (double2 units); [N][P+1]
	int a;		// applications this step (0 = inactive)
};

// ffmap (field-free chains only, optional): the instance whose own field-free factors a chain of
// instance inst uses, at ffmap[inst] * ffstride; without it every instance shares one set.
template <bool CPL>
__device__ __forceinline__ chain_desc describe(long ch, long nchains, const int64_t* __restrict__ nta, long step, int jslot,
	int B, int M, int m0, int N, int L, int np, int NE, const int* __restrict__ ffmap = nullptr, long ffstride = 0, int cmode = 0)
{
	chain_desc d{0, 0, 0};
	if (ch >= nchains) return d;
	if (CPL) {
		long pr = ch >> 1;
		int sign = (int)(ch & 1);
		int k = (int)(pr % np);
		long im_inst = pr / np;
		long inst = im_inst / M;
		d.xoff = im_inst * (long)N * L + 2 * k + sign;
		d.foff = (((long)jslot * B * M + im_inst) * np + k) * (long)N * NE;
		d.a = coupling_power(step, nta[inst], cmode);
	} else {
		int il = (int)(ch % L);
		long im_inst = ch / L;
		int m = (int)(im_inst % M) + m0;
		long inst = im_inst / M;
		int l = il + (m < 0 ? -m : m);
		d.xoff = im_inst * (long)N * L + il;
		d.foff = (long)l * N * NE + (ffmap ? (long)ffmap[inst] * ffstride : 0L);
		d.a = step < nta[inst] ? 1 : 0;
	}
	return d;
}

__device__ __forceinline__ double part_of(double2 v, int part) { return part ? v.y : v.x; }

// operands for acc -= part(l * v) as two FMAs, acc = fma(-l.x, u, fma(l.y, w, acc)):
// real part u = vr, w = vi; imaginary part u = vi, w = -vr (sign flip as an integer op)
__device__ __forceinline__ void msub_operands(double vr, double vi, int part, double& u, double& w)
{
	u = part ? vi : vr;
	w = part ? __longlong_as_double(__double_as_longlong(vr) ^ (long long)0x8000000000000000ull) : vi;
}

// own part of (l * v), complex l and v, as l.x u - l.y w with the operands of msub_operands: the
// same two FP64 instructions on both parts (a select between two FP64 expressions would make a
// warp with both parts issue both)
__device__ __forceinline__ double cmul_part(double2 l, double vr, double vi, int part)
{
	double u, w;
	msub_operands(vr, vi, part, u, w);
	return fma(l.x, u, -l.y * w);
}


// warps per block of k_chain: one staged S band serves every warp of a block (the launch chooses
// 1..CHAIN_MAXW warps; 4 unless the engine is told otherwise)
constexpr int CHAIN_MAXW = 5;

template <int P, int G, bool CPL>
__global__ void __launch_bounds__(CHAIN_MAXW * 32) k_chain(double2* __restrict__ X, double2* __restrict__ Wk,
	const double2* __restrict__ fac, const double* __restrict__ S, const int64_t* __restrict__ nta,
	long step, int jslot, int B, int M, int m0, int N, int L, int np, long chbase, long nchains,
	const double* __restrict__ Fo = nullptr, double* __restrict__ obs = nullptr, const int* __restrict__ ffmap = nullptr, long ffstride = 0,
	int cmode = 0, int sstage = 1)
{
	// chains [chbase, nchains) of this launch (an instance group); nchains is an end index.
	// Fo/obs (coupling chains only, optional): obs[chain] = <z|F|z> of the chain's vector at
	// the point where it represents the wavefunction at t_step -- before the first
	// application at step 0, after the first of two applications otherwise.
	using C = chain_cfg<P, G, CPL>;
	constexpr int NE = C::NE, LPC = C::LPC, CPW = C::CPW, TPL = C::TPL, PD = C::PD;
	// S band [N][P+1]: staged in shared memory per block (sstage), or read through L1, which
	// leaves the shared memory to more resident blocks
	extern __shared__ double sS[];
	const double* Sb = S;
	if (sstage) {
		for (int t = threadIdx.x; t < N * NE; t += blockDim.x) sS[t] = S[t];
		__syncthreads();
		Sb = sS;
	}
	const unsigned FULL = 0xffffffffu;
	const int lane = threadIdx.x & 31;
	const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const long ch0 = chbase + warp * CPW;
	if (ch0 >= nchains) return;
	// chain descriptors of this warp, once, in shared memory
	__shared__ long s_x[CHAIN_MAXW][32], s_f[CHAIN_MAXW][32];
	__shared__ int s_a[CHAIN_MAXW][32];
	const int wib = threadIdx.x >> 5;
	if (lane < CPW) {
		chain_desc d = describe<CPL>(ch0 + lane, nchains, nta, step, jslot, B, M, m0, N, L, np, NE, ffmap, ffstride, cmode);
		s_x[wib][lane] = d.xoff; s_f[wib][lane] = d.foff; s_a[wib][lane] = d.a;
	}
	__syncwarp();
	auto desc = [&](int cl) { chain_desc d; d.xoff = s_x[wib][cl]; d.foff = s_f[wib][cl]; d.a = s_a[wib][cl]; return d; };
	int amax = 0;
#pragma unroll
	for (int cl = 0; cl < CPW; ++cl) amax = max(amax, s_a[wib][cl]);
	if (amax == 0) return;
	double* Xd = reinterpret_cast<double*>(X);
	double* Wd = reinterpret_cast<double*>(Wk);
	const long rs = 2L * L;	// row stride in doubles

	// systolic role of this lane
	const int cls = lane / LPC;
	const int ps = (lane % LPC) / G;
	const int g = lane % G;
	const int cbase = cls * LPC;
	const bool srole = cls < CPW;
	const chain_desc ds = srole ? desc(cls) : chain_desc{0, 0, 0};
	const double2* fs = fac + ds.foff;
	double* ws = Wd + 2 * ds.xoff + ps;

	// observation pass: every lane has a fixed (chain, part) when CPW divides 16
	auto observe = [&](int app, int pos) {
		if constexpr (CPL && (16 % CPW == 0)) {
			double acc = 0.0;
			for (int base = 0; base < N * CPW * 2; base += 32) {
				int it = base + lane;
				int part = it & 1, cl = (it >> 1) % CPW, r = (it >> 1) / CPW;
				if (it < N * CPW * 2) {
					chain_desc d = desc(cl);
					bool on = d.a > 0 && app == 0 && ((pos == 0 && step == 0) || (pos == 1 && d.a == 2));
					if (on) {
						const double* z = Xd + 2 * d.xoff + part;
						double t = 0.0;
#pragma unroll
						for (int k = P; k >= 1; --k)
							if (r - k >= 0) t = fma(__ldg(Fo + (r - k) * NE + k), z[(long)(r - k) * rs], t);
#pragma unroll
						for (int k = 0; k <= P; ++k)
							if (r + k < N) t = fma(__ldg(Fo + r * NE + k), z[(long)(r + k) * rs], t);
						acc = fma(z[(long)r * rs], t, acc);
					}
				}
			}
			// lanes of one chain differ in bit 0 (part) and in the bits above log2(CPW)+1
			for (int mk = 2 * CPW; mk < 32; mk <<= 1) acc += __shfl_xor_sync(FULL, acc, mk);
			acc += __shfl_xor_sync(FULL, acc, 1);
			if (lane < 2 * CPW && !(lane & 1)) {
				int cl = lane >> 1;
				chain_desc d = desc(cl);
				bool on = d.a > 0 && app == 0 && ((pos == 0 && step == 0) || (pos == 1 && d.a == 2));
				if (on) obs[ch0 + cl] = acc;
			}
		}
	};

	for (int app = 0; app < amax; ++app) {
		if (obs && app == 0) { observe(0, 0); __syncwarp(); }
		// ---- P1: w = S z  (items: row r, chain cl, part)
		for (int base = 0; base < N * CPW * 2; base += 32) {
			int it = base + lane;
			int part = it & 1, cl = (it >> 1) % CPW, r = (it >> 1) / CPW;
			if (it < N * CPW * 2) {
				chain_desc d = desc(cl);
				if (app < d.a) {
					const double* z = Xd + 2 * d.xoff + part;
					double w = 0.0;
#pragma unroll
					for (int k = P; k >= 1; --k)
						if (r - k >= 0) w = fma(Sb[(r - k) * NE + k], z[(long)(r - k) * rs], w);
#pragma unroll
					for (int k = 0; k <= P; ++k)
						if (r + k < N) w = fma(Sb[r * NE + k], z[(long)(r + k) * rs], w);
					Wd[2 * d.xoff + part + (long)r * rs] = w;
				}
			}
		}
		__syncwarp();
		const bool act = srole && app < ds.a;
		// ---- P2: y = L^-1 w, column-oriented systolic window (rows c+1+g*TPL+t).
		// The factor entries of column c and the value entering the window are
		// fetched PD columns ahead into a register ring.
		{
			double acc[TPL];
#pragma unroll
			for (int t = 0; t < TPL; ++t) {
				int row = g * TPL + t;
				acc[t] = (act && row < N) ? ws[(long)row * rs] : 0.0;
			}
			double2 lr[PD][TPL];
			double wr[PD];
			auto fetch = [&](int c, double2* l, double& we) {
#pragma unroll
				for (int t = 0; t < TPL; ++t) {
					int j = 1 + g * TPL + t, row = c + j;
					l[t] = (act && row < N) ? fs[(long)row * NE + (j - 1)] : make_double2(0.0, 0.0);
				}
				we = (act && g == G - 1 && c + P < N) ? ws[(long)(c + P) * rs] : 0.0;
			};
#pragma unroll
			for (int d = 0; d < PD; ++d) fetch(d, lr[d], wr[d]);
			for (int c0 = 0; c0 < N; c0 += PD) {
#pragma unroll
				for (int d = 0; d < PD; ++d) {
					const int c = c0 + d;
					if (c >= N) break;
					double yr = __shfl_sync(FULL, acc[0], cbase);
					double yi = __shfl_sync(FULL, acc[0], cbase + G);
					double u, w;
					msub_operands(yr, yi, ps, u, w);
					if (act && g == 0) ws[(long)c * rs] = acc[0];
					double nxt = __shfl_sync(FULL, acc[0], (lane + 1) & 31);
#pragma unroll
					for (int t = 0; t < TPL - 1; ++t) acc[t] = acc[t + 1];
					acc[TPL - 1] = (g == G - 1) ? wr[d] : nxt;
#pragma unroll
					for (int t = 0; t < TPL; ++t) acc[t] = fma(-lr[d][t].x, u, fma(lr[d][t].y, w, acc[t]));
					fetch(c + PD, lr[d], wr[d]);
				}
			}
		}
		__syncwarp();
		// ---- P3: y <- D^-1 y
		for (int base = 0; base < N * CPW * 2; base += 32) {
			int it = base + lane;
			int part = it & 1, cl = (it >> 1) % CPW, r = (it >> 1) / CPW;
			bool v = false;
			double res = 0.0;
			long o = 0;
			if (it < N * CPW * 2) {
				chain_desc d = desc(cl);
				if (app < d.a) {
					o = 2 * d.xoff + (long)r * rs;
					double2 y = make_double2(Wd[o], Wd[o + 1]);
					double2 dv = fac[d.foff + (long)r * NE + P];
					res = cmul_part(dv, y.x, y.y, part);
					v = true;
				}
			}
			__syncwarp();
			if (v) Wd[o + part] = res;
		}
		__syncwarp();
		// ---- P4: x = L^-T y, descending (rows c-1-g*TPL-t), same ring prefetch
		{
			double acc[TPL];
#pragma unroll
			for (int t = 0; t < TPL; ++t) {
				int row = N - 1 - g * TPL - t;
				acc[t] = (act && row >= 0) ? ws[(long)row * rs] : 0.0;
			}
			double2 lr[PD][TPL];
			double wr[PD];
			auto fetch = [&](int c, double2* l, double& we) {
#pragma unroll
				for (int t = 0; t < TPL; ++t) {
					int j = 1 + g * TPL + t, row = c - j;
					l[t] = (act && row >= 0) ? fs[(long)c * NE + (j - 1)] : make_double2(0.0, 0.0);	// L(c, c-j)
				}
				we = (act && g == G - 1 && c - P >= 0) ? ws[(long)(c - P) * rs] : 0.0;
			};
#pragma unroll
			for (int d = 0; d < PD; ++d) fetch(N - 1 - d, lr[d], wr[d]);
			for (int c0 = N - 1; c0 >= 0; c0 -= PD) {
#pragma unroll
				for (int d = 0; d < PD; ++d) {
					const int c = c0 - d;
					if (c < 0) break;
					double xr = __shfl_sync(FULL, acc[0], cbase);
					double xi = __shfl_sync(FULL, acc[0], cbase + G);
					double u, w;
					msub_operands(xr, xi, ps, u, w);
					if (act && g == 0) ws[(long)c * rs] = acc[0];
					double nxt = __shfl_sync(FULL, acc[0], (lane + 1) & 31);
#pragma unroll
					for (int t = 0; t < TPL - 1; ++t) acc[t] = acc[t + 1];
					acc[TPL - 1] = (g == G - 1) ? wr[d] : nxt;
#pragma unroll
					for (int t = 0; t < TPL; ++t) acc[t] = fma(-lr[d][t].x, u, fma(lr[d][t].y, w, acc[t]));
					fetch(c - PD, lr[d], wr[d]);
				}
			}
		}
		__syncwarp();
		// ---- P5: z <- 2x - z; after the last application of a coupling pair, emit
		//      s = z+ + conj(z-bar), d = z+ - conj(z-bar) for the backward transform
		if (CPL) {
			constexpr int PPW = CPW / 2;
			for (int base = 0; base < N * PPW * 2; base += 32) {
				int it = base + lane;
				int part = it & 1, pl = (it >> 1) % PPW, r = (it >> 1) / PPW;
				if (it < N * PPW * 2) {
					chain_desc dp = desc(2 * pl);
					chain_desc dm = desc(2 * pl + 1);
					if (app < dp.a) {
						long op = 2 * dp.xoff + (long)r * rs + part, om = 2 * dm.xoff + (long)r * rs + part;
						double zp = fma(2.0, Wd[op], -Xd[op]);
						double zm = fma(2.0, Wd[om], -Xd[om]);
						if (app + 1 < dp.a) { Xd[op] = zp; Xd[om] = zm; }
						else {
							double zc = part ? -zm : zm;	// conj(z-bar), own part
							Xd[op] = zp + zc;
							Xd[om] = zp - zc;
						}
					}
				}
			}
		} else {
			for (int base = 0; base < N * CPW * 2; base += 32) {
				int it = base + lane;
				int part = it & 1, cl = (it >> 1) % CPW, r = (it >> 1) / CPW;
				if (it < N * CPW * 2) {
					chain_desc d = desc(cl);
					if (app < d.a) {
						long o = 2 * d.xoff + (long)r * rs + part;
						Xd[o] = fma(2.0, Wd[o], -Xd[o]);
					}
				}
			}
		}
		__syncwarp();
		if (obs && app == 0) { observe(0, 1); __syncwarp(); }
	}
}

// ---------------------------------------------------------------- segmented (latency) variant
// For few chains the recurrences P2/P4 are the critical path: one row costs ~650 cycles of dependent
// FP64 work with the GPU otherwise idle.  k_chain_seg cuts each chain into Q segments of Ls rows
// (Ls >= P, last segment >= P rows) and solves them at once (one lane pair per segment), then joins
// them: with y0 the solution of a segment whose history is zero and Phi_j the homogeneous solution
// with a unit value entering from row a - j (forward; b - 1 + j backward), the true values are
// y = y0 + sum_j Phi_j x_j, where x are the last P values of the previous segment -- a chain of Q
// small P x P steps.  The Phi depend only on the factors, so they are computed with them (k_spikes
// for the coupling factors, on the host for the field-free ones).  The two recurrences then take
// ~Ls + Q row times instead of N; every other pass is row-parallel over the block.

// Phi_j (forward, L y = 0 with y_{a-j} = 1 entering) or Psi_j (backward, L^T x = 0 with
// x_{b-1+j} = 1 entering) on rows [a, b) of one factor block (rows [N][P+1], L(r, r-k) at
// [r][k-1]); out[r*P + j - 1].  The same code runs on the host and the device.
template <int P>
__host__ __device__ inline void seg_spike(const double2* fs, int N, int a, int b, int j, bool fwd, double2* out)
{
	constexpr int NE = P + 1;
	if (fwd) {
		for (int r = a; r < b; ++r) {
			double re = 0.0, im = 0.0;
			for (int k = 1; k <= P; ++k) {
				const int src = r - k;
				double2 y;
				if (src >= a) y = out[src * P + j - 1];
				else if (src == a - j && src >= 0) y = make_double2(1.0, 0.0);
				else continue;
				const double2 l = fs[r * NE + k - 1];
				re -= l.x * y.x - l.y * y.y;
				im -= l.x * y.y + l.y * y.x;
			}
			out[r * P + j - 1] = make_double2(re, im);
		}
	} else {
		for (int r = b - 1; r >= a; --r) {
			double re = 0.0, im = 0.0;
			for (int k = 1; k <= P; ++k) {
				const int dst = r + k;
				if (dst >= N) continue;
				double2 x;
				if (dst < b) x = out[dst * P + j - 1];
				else if (dst == b - 1 + j) x = make_double2(1.0, 0.0);
				else continue;
				const double2 l = fs[dst * NE + k - 1];	// L(r+k, r)
				re -= l.x * x.x - l.y * x.y;
				im -= l.x * x.y + l.y * x.x;
			}
			out[r * P + j - 1] = make_double2(re, im);
		}
	}
}

// spikes of the coupling factor blocks [slot < kf][inst b0 .. b0+Bc)[m][pair]: one thread per
// (block, segment, j, direction)
template <int P>
__global__ void k_spikes(const double2* __restrict__ fac, double2* __restrict__ spf, double2* __restrict__ spb, int B, int b0, int Bc,
	int M, int np, int N, int Q, int Ls, long total)
{
	const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= total) return;
	const int dir = (int)(t & 1);
	long u = t >> 1;
	const int j = (int)(u % P); u /= P;
	const int seg = (int)(u % Q); u /= Q;
	const int k = (int)(u % np); u /= np;
	const int m = (int)(u % M); u /= M;
	const int i = (int)(u % Bc);
	const long slot = u / Bc;
	const long blk = ((slot * B + b0 + i) * M + m) * np + k;
	const int a = seg * Ls, b = min(N, a + Ls);
	seg_spike<P>(fac + blk * (long)N * (P + 1), N, a, b, j + 1, dir == 0, (dir == 0 ? spf : spb) + blk * (long)N * P);
}

// One segment's recurrence with zero history, for the forward (L^-1, rows a .. b-1) or the backward
// (L^-T, rows b-1 .. a) solve: lane pair (part 0, 1) of a segment, work vector wv (own part, stride
// 2 doubles), factor rows fs (L(r, r-k) at fs[r (P+1) + k - 1]).  The factor entries and the value
// of the next row are fetched one row ahead.
template <int P, bool FWD>
__device__ __forceinline__ void seg_recurrence(double* wv, const double2* fs, int a, int b, int Ls, bool on, int part)
{
	constexpr int NE = P + 1;
	const unsigned FULL = 0xffffffffu;
	double hr[P], hi[P];
	double2 l[P], ln[P];
#pragma unroll
	for (int k = 0; k < P; ++k) { hr[k] = 0.0; hi[k] = 0.0; l[k] = make_double2(0.0, 0.0); }
	const int r0 = FWD ? a : b - 1;
	double wcur = (on && a < b) ? wv[2L * r0] : 0.0;
	for (int t = 0; t < Ls; ++t) {
		const int r = FWD ? a + t : b - 1 - t;
		const int rn = FWD ? r + 1 : r - 1;
		const bool live = on && t < b - a;
		const bool nlive = on && t + 1 < b - a;
#pragma unroll
		for (int k = 1; k <= P; ++k) {
			const long li = FWD ? (long)rn * NE + (k - 1) : (long)(rn + k) * NE + (k - 1);	// L(rn, rn-k) | L(rn+k, rn)
			ln[k - 1] = (nlive && t + 1 - k >= 0) ? fs[li] : make_double2(0.0, 0.0);
		}
		const double wnext = nlive ? wv[2L * rn] : 0.0;
		double acc = live ? wcur : 0.0;
		// own part of acc - l y with the same two FMAs on both parts (operands chosen by integer
		// selects, so the warp issues no FP64 instruction twice)
#pragma unroll
		for (int k = 0; k < P; ++k) {
			double u, w;
			msub_operands(hr[k], hi[k], part, u, w);
			acc = fma(-l[k].x, u, fma(l[k].y, w, acc));
		}
		const double other = __shfl_xor_sync(FULL, acc, 1);
#pragma unroll
		for (int k = P - 1; k >= 1; --k) { hr[k] = hr[k - 1]; hi[k] = hi[k - 1]; }
		hr[0] = part ? other : acc;
		hi[0] = part ? acc : other;
		if (live) wv[2L * r] = acc;
#pragma unroll
		for (int k = 0; k < P; ++k) l[k] = ln[k];
		wcur = wnext;
	}
}

// threads of a k_chain_seg block: the sequential parts run on one warp per chain, the passes over
// all rows on every warp (8 warps: two per SM sub-partition, to hide the latency of their loads)
constexpr int SEG_THREADS = 256;

// Shared memory of k_chain_seg, in double2 units: the factor block [N][P+1] when SFAC, the work
// vectors [NC][N], and the spike rows the carry chains read, forward [Q][P][P] and backward [Q][P][P].
__host__ __device__ inline long seg_smem_elems(int N, int P, int NC, int Q, bool sfac)
{
	return (sfac ? (long)N * (P + 1) : 0L) + (long)NC * N + 2L * Q * P * P;
}

// One block per chain (field-free) or per (+s, -s) pair (coupling); the same passes as k_chain, with
// the recurrences segmented.  spf/spb: the spikes of every factor block, [block][N][P], block =
// foff / (N (P+1)).  SEG_THREADS threads; segment lanes: warp c handles chain c, lane = 2 segment + part.
// The chain is latency-bound (a few dozen blocks in flight), so everything the sequential parts
// read sits in shared memory: the work vectors always, the rows of the spikes that the carry
// chains read (P per segment boundary), and the factor block when it fits (SFAC); the passes
// over all rows (S z, the fix-ups) read the band and the spikes through L1/L2 in parallel.
template <int P, bool CPL, bool SFAC>
__global__ void __launch_bounds__(SEG_THREADS, 1) k_chain_seg(double2* __restrict__ X, const double2* __restrict__ fac,
	const double2* __restrict__ spf, const double2* __restrict__ spb, const double* __restrict__ S, const int64_t* __restrict__ nta,
	long step, int jslot, int B, int M, int m0, int N, int L, int np, long chbase, long nchains, int Q, int Ls,
	const int* __restrict__ ffmap, long ffstride, int cmode)
{
	constexpr int NE = P + 1, NC = CPL ? 2 : 1;
	static_assert(2 * P <= 16, "carry lanes: 16 h + 2 i + part");
	const unsigned FULL = 0xffffffffu;
	extern __shared__ double2 seg_sm[];
	__shared__ double2 xc[NC][16][P];
	__shared__ long s_x[NC], s_f[NC];
	__shared__ int s_a[NC];
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const long ch0 = chbase + (long)blockIdx.x * NC;
	if (tid < NC) {
		chain_desc d = describe<CPL>(ch0 + tid, nchains, nta, step, jslot, B, M, m0, N, L, np, NE, ffmap, ffstride, cmode);
		s_x[tid] = d.xoff; s_f[tid] = d.foff; s_a[tid] = d.a;
	}
	__syncthreads();
	int amax = 0;
#pragma unroll
	for (int c = 0; c < NC; ++c) amax = max(amax, s_a[c]);
	if (amax == 0) return;	// uniform over the block
	// the chains of a block share one factor block (a (+s, -s) pair uses one LDL^T)
	const double2* fblk = fac + s_f[0];
	const long sblk = (s_f[0] / ((long)N * NE)) * (long)N * P;
	const double2* spfb = spf + sblk;
	const double2* spbb = spb + sblk;
	double2* fsh = seg_sm;
	double2* wsh = seg_sm + (SFAC ? (long)N * NE : 0L);
	double2* cfw = wsh + (long)NC * N;	// [sg][i][jj]: forward spike at row sg Ls - 1 - i, sg = 1 .. Q-1
	double2* cbw = cfw + Q * P * P;	// [sg][i][jj]: backward spike at row (sg + 1) Ls + i, sg = 0 .. Q-2
	if (SFAC) {
		// the factor block, 16-byte asynchronous copies (all in flight at once)
		const uint32_t fbase = (uint32_t)__cvta_generic_to_shared(fsh);
		for (int t = tid; t < N * NE; t += blockDim.x)
			asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(fbase + 16u * (uint32_t)t), "l"(fblk + t));
		asm volatile("cp.async.commit_group;\n" ::);
	}
	for (int t = tid; t < (Q - 1) * P * P; t += blockDim.x) {
		const int jj = t % P, i = (t / P) % P, sg = t / (P * P);
		cfw[((sg + 1) * P + i) * P + jj] = spfb[(long)((sg + 1) * Ls - 1 - i) * P + jj];
		cbw[(sg * P + i) * P + jj] = spbb[(long)((sg + 1) * Ls + i) * P + jj];
	}
	if (SFAC) asm volatile("cp.async.wait_group 0;\n" ::);
	__syncthreads();
	const double2* fs = SFAC ? fsh : fblk;
	double* Xd = reinterpret_cast<double*>(X);
	const long rs = 2L * L;
	for (int app = 0; app < amax; ++app) {
		// ---- P1: w = S z
		for (int it = tid; it < NC * N; it += blockDim.x) {
			const int c = it / N, r = it % N;
			if (app < s_a[c]) {
				const double* z = Xd + 2 * s_x[c];
				double wr = 0.0, wi = 0.0;
#pragma unroll
				for (int k = P; k >= 1; --k)
					if (r - k >= 0) { const double sv = __ldg(S + (r - k) * NE + k); wr = fma(sv, z[(long)(r - k) * rs], wr); wi = fma(sv, z[(long)(r - k) * rs + 1], wi); }
#pragma unroll
				for (int k = 0; k <= P; ++k)
					if (r + k < N) { const double sv = __ldg(S + r * NE + k); wr = fma(sv, z[(long)(r + k) * rs], wr); wi = fma(sv, z[(long)(r + k) * rs + 1], wi); }
				wsh[c * N + r] = make_double2(wr, wi);
			}
		}
		__syncthreads();
		// ---- P2a: y0 = L^-1 w per segment (zero history), lane = 2 segment + part
		if (warp < NC) {
			const int c = warp, seg = lane >> 1, part = lane & 1;
			const int a0 = seg * Ls, b0 = min(N, a0 + Ls);
			seg_recurrence<P, true>(reinterpret_cast<double*>(wsh + c * N) + part, fs, a0, b0, Ls, app < s_a[c] && seg < Q, part);
		}
		__syncthreads();
		// ---- P2b: forward carries x(s)_i = y(a_s - 1 - i), s = 1..Q-1.  lane = 16 h + 2 i + part: the
		// two halves h of the sum over j run on separate lanes (two FMAs per term) and are joined by
		// one shuffle, so a carry step costs ceil(P/2) * 2 + 1 FP64 instructions
		if (warp < NC) {
			constexpr int HJ = (P + 1) / 2;
			const int c = warp, h = lane >> 4, i = (lane & 15) >> 1, part = lane & 1;
			const bool on = app < s_a[c] && i < P;
			const double* wv = reinterpret_cast<const double*>(wsh + c * N) + part;
			for (int sg = 1; sg < Q; ++sg) {
				double v = 0.0;
				if (on) {
					const int r = sg * Ls - 1 - i;
					if (h == 0) v = wv[2L * r];
					if (sg >= 2) {
#pragma unroll
						for (int q = 0; q < HJ; ++q) {
							const int jj = h * HJ + q;
							if (jj < P) {
								const double2 ph = cfw[(sg * P + i) * P + jj], xv = xc[c][sg - 1][jj];
								double u, w;
								msub_operands(xv.x, xv.y, part, u, w);	// own part of ph xv = ph.x u - ph.y w
								v = fma(ph.x, u, fma(-ph.y, w, v));
							}
						}
					}
				}
				v += __shfl_xor_sync(FULL, v, 16);
				__syncwarp();
				if (on && h == 0) reinterpret_cast<double*>(&xc[c][sg][i])[part] = v;
				__syncwarp();
			}
		}
		__syncthreads();
		// ---- P2c + P3: y = y0 + sum_j Phi_j x(s)_j, then y <- D^-1 y
		for (int it = tid; it < NC * N; it += blockDim.x) {
			const int c = it / N, r = it % N;
			if (app < s_a[c]) {
				const int sg = r / Ls;
				double2 y = wsh[c * N + r];
				if (sg >= 1) {
					const double2* sp = spfb + (long)r * P;
#pragma unroll
					for (int jj = 0; jj < P; ++jj) {
						const double2 ph = __ldg(sp + jj), xv = xc[c][sg][jj];
						y.x += ph.x * xv.x - ph.y * xv.y;
						y.y += ph.x * xv.y + ph.y * xv.x;
					}
				}
				const double2 dv = fs[(long)r * NE + P];
				wsh[c * N + r] = make_double2(dv.x * y.x - dv.y * y.y, dv.x * y.y + dv.y * y.x);
			}
		}
		__syncthreads();
		// ---- P4a: x0 = L^-T y per segment (zero history above), descending
		if (warp < NC) {
			const int c = warp, seg = lane >> 1, part = lane & 1;
			const int a0 = seg * Ls, b0 = min(N, a0 + Ls);
			seg_recurrence<P, false>(reinterpret_cast<double*>(wsh + c * N) + part, fs, a0, b0, Ls, app < s_a[c] && seg < Q, part);
		}
		__syncthreads();
		// ---- P4b: backward carries x(s)_i = x(b_s + i), s = Q-2 .. 0, lanes as in P2b
		if (warp < NC) {
			constexpr int HJ = (P + 1) / 2;
			const int c = warp, h = lane >> 4, i = (lane & 15) >> 1, part = lane & 1;
			const bool on = app < s_a[c] && i < P;
			const double* wv = reinterpret_cast<const double*>(wsh + c * N) + part;
			for (int sg = Q - 2; sg >= 0; --sg) {
				double v = 0.0;
				if (on) {
					const int r = (sg + 1) * Ls + i;
					if (h == 0) v = wv[2L * r];
					if (sg + 1 <= Q - 2) {
#pragma unroll
						for (int q = 0; q < HJ; ++q) {
							const int jj = h * HJ + q;
							if (jj < P) {
								const double2 ph = cbw[(sg * P + i) * P + jj], xv = xc[c][sg + 1][jj];
								double u, w;
								msub_operands(xv.x, xv.y, part, u, w);	// own part of ph xv = ph.x u - ph.y w
								v = fma(ph.x, u, fma(-ph.y, w, v));
							}
						}
					}
				}
				v += __shfl_xor_sync(FULL, v, 16);
				__syncwarp();
				if (on && h == 0) reinterpret_cast<double*>(&xc[c][sg][i])[part] = v;
				__syncwarp();
			}
		}
		__syncthreads();
		// ---- P4c + P5: x = x0 + sum_j Psi_j x(s)_j, then z <- 2x - z (pairs: s/d emission after the last application)
		for (int r = tid; r < N; r += blockDim.x) {
			const int sg = r / Ls;
			double xr[NC], xi[NC];
#pragma unroll
			for (int c = 0; c < NC; ++c) {
				xr[c] = 0.0; xi[c] = 0.0;
				if (app < s_a[c]) {
					const double2 w0 = wsh[c * N + r];
					xr[c] = w0.x; xi[c] = w0.y;
					if (sg <= Q - 2) {
						const double2* sp = spbb + (long)r * P;
#pragma unroll
						for (int jj = 0; jj < P; ++jj) {
							const double2 ph = __ldg(sp + jj), xv = xc[c][sg][jj];
							xr[c] += ph.x * xv.x - ph.y * xv.y;
							xi[c] += ph.x * xv.y + ph.y * xv.x;
						}
					}
				}
			}
			if (CPL) {
				if (app < s_a[0]) {
					const long op = 2 * s_x[0] + (long)r * rs, om = 2 * s_x[NC - 1] + (long)r * rs;
					const double zpr = fma(2.0, xr[0], -Xd[op]), zpi = fma(2.0, xi[0], -Xd[op + 1]);
					const double zmr = fma(2.0, xr[NC - 1], -Xd[om]), zmi = fma(2.0, xi[NC - 1], -Xd[om + 1]);
					if (app + 1 < s_a[0]) { Xd[op] = zpr; Xd[op + 1] = zpi; Xd[om] = zmr; Xd[om + 1] = zmi; }
					else {	// conj(z-bar) = (zmr, -zmi)
						Xd[op] = zpr + zmr; Xd[op + 1] = zpi - zmi;
						Xd[om] = zpr - zmr; Xd[om + 1] = zpi + zmi;
					}
				}
			} else if (app < s_a[0]) {
				const long o = 2 * s_x[0] + (long)r * rs;
				Xd[o] = fma(2.0, xr[0], -Xd[o]);
				Xd[o + 1] = fma(2.0, xi[0], -Xd[o + 1]);
			}
		}
		__syncthreads();
	}
}

} // namespace qpc
