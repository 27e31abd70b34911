// Host side of the slice-product FP64 GEMM (qpc_ozaki.cuh): splitting an operand into its digit
// slices, the product, and qpc_dgemm_slices, the C ABI form on host buffers.
#include "qpc_internal.h"
#include "qpc_cuda_util.cuh"
#include "qpc_ozaki.cuh"
#include "qpc_tcgen05.cuh"
#include <cuda_runtime.h>
#include <cuda.h>
#include <vector>
#include <cstdlib>

namespace qpc {
namespace oz {

__device__ __forceinline__ const double* elem(const operand& o, long k, long j)
{
	const long q = j / o.jdiv, r = j - q * o.jdiv;
	return o.p + q * o.jouter + r * o.jstride + k * o.kstride;
}

// biased exponent field of the largest |x| over k of every column j: ef[j] = max (bits >> 52) & 0x7ff
// (ef must start at 0); blocks of 256 columns x KR rows
__global__ void k_oz_exp(operand o, long K, long J, int* __restrict__ ef)
{
	const long j = (long)blockIdx.x * 256 + threadIdx.x;
	if (j >= J) return;
	const long k0 = (long)blockIdx.y * EXP_KR;
	const long k1 = k0 + EXP_KR < K ? k0 + EXP_KR : K;
	int m = 0;
	for (long k = k0; k < k1; ++k) {
		const long long b = __double_as_longlong(*elem(o, k, j));
		m = max(m, (int)((b >> 52) & 0x7ff));
	}
	if (m) atomicMax(ef + j, m);
}

// the NS digit slices of every element: D[s][j][k] (k contiguous, row length Kp, zero past K),
// through a 32 x 32 shared-memory tile (reads follow j, writes follow k); block 32 x 8
__global__ void k_oz_split(operand o, long K, long J, long Kp, const int* __restrict__ ef, __nv_bfloat16* __restrict__ D)
{
	__shared__ long long tile[32][33];
	const long j0 = (long)blockIdx.x * 32, k0 = (long)blockIdx.y * 32;
	const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
	for (int r = 0; r < 4; ++r) {
		const long k = k0 + ty + 8 * r, j = j0 + tx;
		tile[ty + 8 * r][tx] = (k < K && j < J) ? __double_as_longlong(*elem(o, k, j)) : 0ll;
	}
	__syncthreads();
	const long sstride = J * Kp;
#pragma unroll
	for (int r = 0; r < 4; ++r) {
		const long j = j0 + ty + 8 * r, k = k0 + tx;
		if (j >= J || k >= Kp) continue;
		const long long b = tile[tx][ty + 8 * r];
		const int fe = (int)((b >> 52) & 0x7ff);
		unsigned long long m = (unsigned long long)b & 0xfffffffffffffull;
		int E = -1022;
		if (fe) { m |= 1ull << 52; E = fe - 1023; }
		const int ejf = ef[j];
		const int ej = ejf ? ejf - 1022 : -1022;
		// Y = trunc(|x| 2^(63 - ej)) = m 2^(E - 52 + 63 - ej) < 2^63
		const int sh = E + 11 - ej;
		unsigned long long Y = 0;
		if (sh >= 0) Y = m << sh;
		else if (sh > -64) Y = m >> (-sh);
		const bool neg = b < 0;
		__nv_bfloat16* d = D + j * Kp + k;
#pragma unroll
		for (int s = 0; s < NS; ++s) {
			const int a = (int)((Y >> (BITS * (NS - 1 - s))) & 127u);
			d[s * sstride] = __int2bfloat16_rn(neg ? -a : a);
		}
	}
}

// digit pairs (s, t) with s + t < NS in order of their level d = s + t: the levels 0..3 (the first
// LOPAIR pairs) and 4..NS-1 are summed by separate launches, each with one int64 accumulator
struct pair_table {
	unsigned char s[NS * (NS + 1) / 2], t[NS * (NS + 1) / 2];
};
__host__ __device__ constexpr pair_table make_pairs()
{
	pair_table p{};
	int q = 0;
	for (int d = 0; d < NS; ++d)
		for (int s = 0; s <= d; ++s) { p.s[q] = (unsigned char)s; p.t[q] = (unsigned char)(d - s); ++q; }
	return p;
}
constexpr int NPAIR = NS * (NS + 1) / 2;
constexpr int LOPAIR = 10;	// pairs of levels 0..3
__constant__ pair_table c_pairs = make_pairs();

// the product's pipeline: one stage holds a 64 x 64 digit tile of A (rows of the output tile, 64
// values of k) and one of B; 16-byte chunks of a tile row are stored at chunk ^ (row & 7) so that
// ldmatrix reads 8 rows without bank conflicts
constexpr int KS = 64, NSTAGE = 4;
constexpr int STAGE_ELEMS = 2 * TM * KS;	// bf16 per stage (A tile, then B tile)
constexpr size_t GEMM_SMEM = sizeof(__nv_bfloat16) * STAGE_ELEMS * NSTAGE;

using tc::smem_u32;

// 16 bytes global -> shared, zero-filled when !valid
__device__ __forceinline__ void cp16(uint32_t dst, const void* src, bool valid)
{
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0));
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3)
{
	asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n" : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(addr));
}

// position of the product: digit pair p, exact-sum chunk starting at kc0, stage k offset k0
struct cursor {
	int p;
	long kc0, k0;
};

__device__ __forceinline__ void advance(cursor& c, long Kp)
{
	c.k0 += KS;
	const long kc1 = c.kc0 + KC < Kp ? c.kc0 + KC : Kp;
	if (c.k0 >= kc1) {
		c.kc0 += KC;
		if (c.kc0 >= Kp) { c.kc0 = 0; ++c.p; }
		c.k0 = c.kc0;
	}
}

// out(i, j) = sum_k A(i, k) B(k, j) for i < n, j < M from the digit slices Da [NS][n][Kp] and
// Db [NS][M][Kp] and the exponent fields ea [n], eb [M]; out(i, j) at
// out + (j / jdiv) * jouter + i * istride + (j % jdiv).  128 threads, output tile 64 x 64 (warps
// 2 x 2 of 32 x 32), NSTAGE-deep cp.async pipeline over the (pair, chunk, k) stages.
// HI = true: the pairs of levels 0..3, their exact sum (units of 2^-35) stored to hsum [n][M];
// HI = false: the pairs of levels 4..NS-1 (units of 2^-70), combined with hsum into out.
template <bool HI>
__global__ void __launch_bounds__(THREADS) k_oz_gemm(const __nv_bfloat16* __restrict__ Da, const int* __restrict__ ea,
	const __nv_bfloat16* __restrict__ Db, const int* __restrict__ eb, long n, long M, long Kp, long long* __restrict__ hsum,
	double* __restrict__ out, long istride, long jdiv, long jouter)
{
	constexpr int P0 = HI ? 0 : LOPAIR, P1 = HI ? LOPAIR : NPAIR;
	extern __shared__ __align__(128) __nv_bfloat16 sm[];
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int gid = lane >> 2, tig = lane & 3;
	const long rowA0 = (long)blockIdx.y * TM, rowB0 = (long)blockIdx.x * TN;
	const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
	const long sa = n * Kp, sb = M * Kp;
	const uint32_t sbase = smem_u32(sm);

	// producer: stage of cursor c into slot
	auto load_stage = [&](const cursor& c, int slot) {
		if (c.p >= P1) return;
		const long kc1 = c.kc0 + KC < Kp ? c.kc0 + KC : Kp;
		const __nv_bfloat16* A = Da + (long)c_pairs.s[c.p] * sa;
		const __nv_bfloat16* B = Db + (long)c_pairs.t[c.p] * sb;
		const uint32_t dA = sbase + (uint32_t)(slot * STAGE_ELEMS) * 2u, dB = dA + (uint32_t)(TM * KS) * 2u;
#pragma unroll
		for (int u = 0; u < 4; ++u) {
			const int idx = tid + THREADS * u;
			const int r = idx >> 3, ch = idx & 7;
			const long k = c.k0 + ch * 8;
			const uint32_t off = (uint32_t)(r * 128 + ((ch ^ (r & 7)) << 4));
			const bool kin = k < kc1;
			const long ra = rowA0 + r, rb = rowB0 + r;
			cp16(dA + off, A + (ra < n && kin ? ra * Kp + k : 0), ra < n && kin);
			cp16(dB + off, B + (rb < M && kin ? rb * Kp + k : 0), rb < M && kin);
		}
	};

	long long isum[2][4][4];
	float acc[2][4][4];
#pragma unroll
	for (int i = 0; i < 2; ++i)
#pragma unroll
		for (int j = 0; j < 4; ++j)
#pragma unroll
			for (int q = 0; q < 4; ++q) { isum[i][j][q] = 0; acc[i][j][q] = 0.f; }

	cursor prod{P0, 0, 0}, cons{P0, 0, 0};
#pragma unroll
	for (int st = 0; st < NSTAGE - 1; ++st) {
		load_stage(prod, st);
		asm volatile("cp.async.commit_group;\n" ::);
		advance(prod, Kp);
	}
	int slot = 0;
	while (cons.p < P1) {
		asm volatile("cp.async.wait_group %0;\n" ::"n"(NSTAGE - 2));
		__syncthreads();
		// refill the slot consumed in the previous iteration
		load_stage(prod, (slot + NSTAGE - 1) % NSTAGE);
		asm volatile("cp.async.commit_group;\n" ::);
		advance(prod, Kp);
		const uint32_t tA = sbase + (uint32_t)(slot * STAGE_ELEMS) * 2u, tB = tA + (uint32_t)(TM * KS) * 2u;
#pragma unroll
		for (int kk = 0; kk < KS / 16; ++kk) {
			uint32_t af[2][4], bfr[4][2];
#pragma unroll
			for (int i = 0; i < 2; ++i) {
				const int mi = lane >> 3;
				const int r = wm + i * 16 + (mi & 1) * 8 + (lane & 7);
				const int ch = kk * 2 + (mi >> 1);
				ldsm_x4(tA + (uint32_t)(r * 128 + ((ch ^ (r & 7)) << 4)), af[i][0], af[i][1], af[i][2], af[i][3]);
			}
#pragma unroll
			for (int jj = 0; jj < 2; ++jj) {
				const int mi = lane >> 3;
				const int r = wn + jj * 16 + (mi >> 1) * 8 + (lane & 7);
				const int ch = kk * 2 + (mi & 1);
				ldsm_x4(tB + (uint32_t)(r * 128 + ((ch ^ (r & 7)) << 4)), bfr[2 * jj][0], bfr[2 * jj][1], bfr[2 * jj + 1][0], bfr[2 * jj + 1][1]);
			}
#pragma unroll
			for (int i = 0; i < 2; ++i)
#pragma unroll
				for (int j = 0; j < 4; ++j)
					asm volatile(
						"mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
						: "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
						: "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bfr[j][0]), "r"(bfr[j][1]));
		}
		// end of an exact-sum chunk of a pair: its integer sums into the level accumulators
		const int p = cons.p;
		advance(cons, Kp);
		if (cons.p != p || cons.k0 == cons.kc0) {
			const int d = c_pairs.s[p] + c_pairs.t[p];
			const int sh = d <= 3 ? BITS * (3 - d) : BITS * (NS - 1 - d);
#pragma unroll
			for (int i = 0; i < 2; ++i)
#pragma unroll
				for (int j = 0; j < 4; ++j)
#pragma unroll
					for (int q = 0; q < 4; ++q) {
						isum[i][j][q] += (long long)__float2int_rn(acc[i][j][q]) << sh;
						acc[i][j][q] = 0.f;
					}
		}
		slot = (slot + 1) % NSTAGE;
	}
	asm volatile("cp.async.wait_group 0;\n" ::);
	// c = 2^(ea + eb) (hi 2^-35 + lo 2^-70); element (row, col) as in the mma accumulator layout
	static_assert(BITS * (NS + 1) == 70 && BITS * 5 == 35, "level scales");
#pragma unroll
	for (int i = 0; i < 2; ++i)
#pragma unroll
		for (int j = 0; j < 4; ++j)
#pragma unroll
			for (int q = 0; q < 4; ++q) {
				const long row = rowA0 + wm + i * 16 + gid + 8 * (q >> 1);
				const long col = rowB0 + wn + j * 8 + tig * 2 + (q & 1);
				if (row >= n || col >= M) continue;
				if (HI) { hsum[row * M + col] = isum[i][j][q]; continue; }
				const long long hi = hsum[row * M + col], lo = isum[i][j][q];
				const int ef_a = ea[row], ef_b = eb[col];
				const int e = (ef_a ? ef_a - 1022 : -1022) + (ef_b ? ef_b - 1022 : -1022);
				// the exact total T = hi 2^35 + lo (units of 2^-70) as th 2^30 + tl with both parts
				// exact in FP64 (|th| < 2^53 for K <= 4096, 0 <= tl < 2^30): one rounding, in the fma
				const long long th = hi * 32 + (lo >> 30);
				const long long tl = lo & ((1ll << 30) - 1);
				const double v = fma((double)th, 0x1p-40, (double)tl * 0x1p-70);
				const long qq = col / jdiv, rr = col - qq * jdiv;
				out[qq * jouter + row * istride + rr] = scalbn(v, e);
			}
}

// ---------------------------------------------------------------- tcgen05 form of the product
// The same digit-pair products on the 5th-generation tensor cores: one thread issues
// tcgen05.mma.cta_group::1.kind::f16 (bf16 x bf16 -> fp32, M = 128, N = 64, K = 16) on operand tiles
// in shared memory (the 128-byte-swizzled K-major layout that cp.async writes: 16-byte chunk c of row r
// at c ^ (r & 7), 8-row groups 1024 bytes apart); the fp32 accumulator of an output tile lives in 64
// columns of tensor memory.  Each stage's MMAs are committed to that stage's mbarrier, which frees the
// stage for the next cp.async refill.  At the end of an exact-sum chunk every thread reads its output
// row from tensor memory (tcgen05.ld) into its int64 level accumulators, and the next chunk starts the
// accumulator afresh.  Every mbarrier wait is bounded: a wait that runs out sets *err and the kernel
// finishes without waiting further (the host reports QPC_ERR_TIMEOUT).
// tile 128 x 128 (M x N), 8 warps: warps w and w + 4 read the tensor-memory lanes 32 (w % 4) .. + 31,
// columns 64 (w / 4) .. + 63, so a thread holds 64 outputs of one row; 6 stages of 32 KB, one CTA per SM
constexpr int TC_M = 128, TC_N = 128, TC_KS = 64, TC_NST = 6, TC_THREADS = 256, TC_COLS_T = 64;
constexpr uint32_t TC_A_BYTES = TC_M * TC_KS * 2, TC_B_BYTES = TC_N * TC_KS * 2, TC_STAGE_BYTES = TC_A_BYTES + TC_B_BYTES;
constexpr uint32_t TC_TMEM_COLS = 128;
constexpr size_t TC_SMEM = (size_t)TC_STAGE_BYTES * TC_NST + 1024 + 8 * TC_NST + 16;
constexpr uint32_t TC_IDESC = tc::idesc_bf16(TC_M, TC_N);
using tc::sw128_desc;
using tc::mbar_init;
using tc::mbar_wait;
__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
	tc::mma_bf16(tmem, adesc, bdesc, TC_IDESC, accumulate);
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) { tc::commit(mbar); }
__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t (&v)[32]) { tc::ld32(taddr, v); }

template <bool HI>
__global__ void __launch_bounds__(TC_THREADS, 1) k_oz_gemm_tc(const __nv_bfloat16* __restrict__ Da, const int* __restrict__ ea,
	const __nv_bfloat16* __restrict__ Db, const int* __restrict__ eb, long n, long M, long Kp, long long* __restrict__ hsum,
	double* __restrict__ out, long istride, long jdiv, long jouter, int* __restrict__ err)
{
	constexpr int P0 = HI ? 0 : LOPAIR, P1 = HI ? LOPAIR : NPAIR;
	extern __shared__ __align__(1024) unsigned char tsm[];
	const uint32_t sraw = smem_u32(tsm);
	const uint32_t sbase = (sraw + 1023u) & ~1023u;	// stages at 1024-byte boundaries (the swizzle's period)
	const uint32_t bars = sbase + TC_STAGE_BYTES * TC_NST;	// TC_NST mbarriers, then the tensor-memory address
	const uint32_t tslot = bars + 8 * TC_NST;
	const int tid = threadIdx.x, warp = tid >> 5;
	const long rowA0 = (long)blockIdx.y * TC_M, rowB0 = (long)blockIdx.x * TC_N;
	const long sa = n * Kp, sb = M * Kp;

	if (tid == 0) {
		for (int q = 0; q < TC_NST; ++q) mbar_init(bars + 8 * q, 1);
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tslot), "r"(TC_TMEM_COLS) : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
	uint32_t tmem;
	asm volatile("ld.shared.u32 %0, [%1];\n" : "=r"(tmem) : "r"(tslot) : "memory");

	// this thread's copies, fixed for the whole tile: rows r_u = tid / 8 + 32 u of A and of B (u < 4),
	// 16-byte chunk ch = tid % 8 of each row's 64-wide k window; source offsets without the slice and
	// the stage's k, destinations within a stage (r_u % 8 is the same for every u)
	const int ch = tid & 7, r0 = tid >> 3;
	const uint32_t dofs = (uint32_t)(r0 * 128 + ((ch ^ (r0 & 7)) << 4));
	// (32-bit: a slice holds fewer than 2^31 digits, checked by the host)
	constexpr int RSTEP = TC_THREADS / 8, UA = TC_M / RSTEP, UB = TC_N / RSTEP;
	uint32_t srcA[UA], srcB[UB];
	unsigned okA = 0, okB = 0;
#pragma unroll
	for (int u = 0; u < UA; ++u) {
		const long row = rowA0 + r0 + RSTEP * u;
		srcA[u] = (uint32_t)((row < n ? row : 0) * Kp + ch * 8);
		okA |= (row < n ? 1u : 0u) << u;
	}
#pragma unroll
	for (int u = 0; u < UB; ++u) {
		const long row = rowB0 + r0 + RSTEP * u;
		srcB[u] = (uint32_t)((row < M ? row : 0) * Kp + ch * 8);
		okB |= (row < M ? 1u : 0u) << u;
	}
	auto load_stage = [&](const cursor& c, int slot) {
		if (c.p >= P1) return;
		const long kc1 = c.kc0 + KC < Kp ? c.kc0 + KC : Kp;
		const bool kin = c.k0 + ch * 8 < kc1;
		const __nv_bfloat16* A = Da + (long)c_pairs.s[c.p] * sa + c.k0;
		const __nv_bfloat16* B = Db + (long)c_pairs.t[c.p] * sb + c.k0;
		const uint32_t dA = sbase + (uint32_t)slot * TC_STAGE_BYTES + dofs, dB = dA + TC_A_BYTES;
#pragma unroll
		for (int u = 0; u < UA; ++u) {
			const bool v = kin && ((okA >> u) & 1u);
			cp16(dA + (uint32_t)(u * RSTEP * 128), v ? A + srcA[u] : Da, v);
		}
#pragma unroll
		for (int u = 0; u < UB; ++u) {
			const bool v = kin && ((okB >> u) & 1u);
			cp16(dB + (uint32_t)(u * RSTEP * 128), v ? B + srcB[u] : Db, v);
		}
	};

	long long isum[TC_COLS_T];
#pragma unroll
	for (int j = 0; j < TC_COLS_T; ++j) isum[j] = 0;
	// stage i is loaded TC_LD stages ahead into the slot of stage i - TC_MD, whose MMAs (committed
	// TC_MD iterations earlier) must be done: loads TC_LD deep, MMAs TC_MD deep (measured: 1 and
	// TC_NST - 1 beat 2 and TC_NST - 2, the loads are what the kernel waits for)
	constexpr int TC_MD = 1, TC_LD = TC_NST - TC_MD;
	cursor prod{P0, 0, 0}, cons{P0, 0, 0};
#pragma unroll
	for (int q = 0; q < TC_LD; ++q) {
		load_stage(prod, q);
		asm volatile("cp.async.commit_group;\n" ::);
		advance(prod, Kp);
	}
	uint32_t parity = 0, pending = 0;	// per stage: phase parity to wait for, commit not yet waited for
	bool fresh = true, ok = true;
	int slot = 0;
	const int lq = warp & 3, cbase = (warp >> 2) * TC_COLS_T;	// lane quarter and first column of this warp
	const uint32_t trow = tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)cbase;
	while (cons.p < P1) {
		asm volatile("cp.async.wait_group %0;\n" ::"n"(TC_LD - 1));
		asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");	// cp.async data -> the tensor core's view
		// the block stops together when any thread's wait ran out (no further MMA is issued)
		if (__syncthreads_or(ok ? 0 : 1)) break;
		asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
		if (tid == 0) {
			const uint32_t aS = sbase + (uint32_t)slot * TC_STAGE_BYTES, bS = aS + TC_A_BYTES;
#pragma unroll
			for (int kk = 0; kk < TC_KS / 16; ++kk)
				tc_mma(tmem, sw128_desc(aS + 32u * kk), sw128_desc(bS + 32u * kk), (fresh && kk == 0) ? 0u : 1u);
			tc_commit(bars + 8 * slot);
		}
		pending |= 1u << slot;
		fresh = false;
		// refill the slot of stage i - TC_MD (stage i + TC_LD goes there) once its MMAs are done
		const int prev = (slot + TC_NST - TC_MD) % TC_NST;
		if (pending & (1u << prev)) {
			if (ok && !mbar_wait(bars + 8 * prev, (parity >> prev) & 1u)) { ok = false; atomicExch(err, 1); }
			parity ^= 1u << prev;
			pending &= ~(1u << prev);
		}
		load_stage(prod, prev);
		asm volatile("cp.async.commit_group;\n" ::);
		advance(prod, Kp);
		// end of an exact-sum chunk: the accumulator into the level sums, the next chunk starts afresh
		const int p = cons.p;
		advance(cons, Kp);
		if (cons.p != p || cons.k0 == cons.kc0) {
			if (ok && !mbar_wait(bars + 8 * slot, (parity >> slot) & 1u)) { ok = false; atomicExch(err, 1); }
			parity ^= 1u << slot;
			pending &= ~(1u << slot);
			asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
			const int d = c_pairs.s[p] + c_pairs.t[p];
			const int sh = d <= 3 ? BITS * (3 - d) : BITS * (NS - 1 - d);
			__syncwarp();	// tcgen05.ld is .sync.aligned: the warp converged
#pragma unroll
			for (int h = 0; h < TC_COLS_T / 32; ++h) {
				uint32_t v[32];
				tc_ld32(trow + 32u * h, v);
#pragma unroll
				for (int j = 0; j < 32; ++j) isum[32 * h + j] += (long long)__float2int_rn(__uint_as_float(v[j])) << sh;
			}
			asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
			fresh = true;
		}
		slot = (slot + 1) % TC_NST;
	}
	asm volatile("cp.async.wait_group 0;\n" ::);
	// MMAs still in flight after a wait ran out: wait for their commits (bounded) before the tensor
	// memory is freed
	for (int q = 0; q < TC_NST; ++q)
		if (pending & (1u << q)) mbar_wait(bars + 8 * q, (parity >> q) & 1u);
	// row i of the tile is tensor-memory lane i: thread (warp, lane) holds output row 32 (warp % 4) + lane,
	// columns cbase .. cbase + 63
	const long row = rowA0 + lq * 32 + (tid & 31);
	if (row < n) {
		const int ef_a = ea[row];
#pragma unroll
		for (int j = 0; j < TC_COLS_T; ++j) {
			const long col = rowB0 + cbase + j;
			if (col >= M) continue;
			if (HI) { hsum[row * M + col] = isum[j]; continue; }
			const long long hi = hsum[row * M + col], lo = isum[j];
			const int ef_b = eb[col];
			const int e = (ef_a ? ef_a - 1022 : -1022) + (ef_b ? ef_b - 1022 : -1022);
			const long long th = hi * 32 + (lo >> 30);
			const long long tl = lo & ((1ll << 30) - 1);
			const double v = fma((double)th, 0x1p-40, (double)tl * 0x1p-70);
			const long qq = col / jdiv, rr = col - qq * jdiv;
			out[qq * jouter + row * istride + rr] = scalbn(v, e);
		}
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
	__syncthreads();
	__syncwarp();
	if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
}

// ---------------------------------------------------------------- tcgen05 with TMA operand loads
// As k_oz_gemm_tc, but the operand tiles arrive by TMA (cp.async.bulk.tensor.2d into the same
// 128-byte-swizzled layout, the tensor maps' swizzle mode), issued by one thread with the stage's
// byte count on its "full" mbarrier; that thread also waits for the data and issues the MMAs, and the
// other warps take part only at the end of an exact-sum chunk (the tensor-memory epilogue).  Rows
// of a tile past the end of a slice read the next slice's rows (their outputs are discarded) or, past
// the array, zeros; no stage crosses an exact-sum chunk (KC is a multiple of TC_KS).
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar)
{
	asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n"
		::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar) : "memory");
}

constexpr size_t TMA_SMEM = (size_t)TC_STAGE_BYTES * TC_NST + 1024 + 16 * TC_NST + 16;

template <bool HI>
__global__ void __launch_bounds__(TC_THREADS, 1) k_oz_gemm_tma(const __grid_constant__ CUtensorMap mapA,
	const __grid_constant__ CUtensorMap mapB, const int* __restrict__ ea, const int* __restrict__ eb, long n, long M, long Kp,
	long long* __restrict__ hsum, double* __restrict__ out, long istride, long jdiv, long jouter, int* __restrict__ err)
{
	constexpr int P0 = HI ? 0 : LOPAIR, P1 = HI ? LOPAIR : NPAIR;
	extern __shared__ __align__(1024) unsigned char tsm[];
	const uint32_t sraw = smem_u32(tsm);
	const uint32_t sbase = (sraw + 1023u) & ~1023u;
	const uint32_t mbars = sbase + TC_STAGE_BYTES * TC_NST;	// MMA-done barriers [TC_NST]
	const uint32_t fbars = mbars + 8 * TC_NST;	// data-arrived barriers [TC_NST]
	const uint32_t tslot = fbars + 8 * TC_NST;
	const int tid = threadIdx.x, warp = tid >> 5;
	const bool leader = tid == 0;
	const long rowA0 = (long)blockIdx.y * TC_M, rowB0 = (long)blockIdx.x * TC_N;

	if (leader) {
		for (int q = 0; q < TC_NST; ++q) { mbar_init(mbars + 8 * q, 1); mbar_init(fbars + 8 * q, 1); }
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
		asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
		asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&mapB)) : "memory");
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tslot), "r"(TC_TMEM_COLS) : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
	uint32_t tmem;
	asm volatile("ld.shared.u32 %0, [%1];\n" : "=r"(tmem) : "r"(tslot) : "memory");

	auto issue_stage = [&](const cursor& c, int slot) {
		if (c.p >= P1) return;
		const uint32_t dA = sbase + (uint32_t)slot * TC_STAGE_BYTES;
		mbar_expect_tx(fbars + 8 * slot, TC_STAGE_BYTES);
		tma_load_2d(dA, &mapA, (int)c.k0, (int)(c_pairs.s[c.p] * n + rowA0), fbars + 8 * slot);
		tma_load_2d(dA + TC_A_BYTES, &mapB, (int)c.k0, (int)(c_pairs.t[c.p] * M + rowB0), fbars + 8 * slot);
	};

	long long isum[TC_COLS_T];
#pragma unroll
	for (int j = 0; j < TC_COLS_T; ++j) isum[j] = 0;
	cursor prod{P0, 0, 0}, cons{P0, 0, 0};
	if (leader)
		for (int q = 0; q < TC_NST - 1; ++q) { issue_stage(prod, q); advance(prod, Kp); }
	uint32_t fpar = 0, mpar = 0, pending = 0;
	bool fresh = true, ok = true;
	int slot = 0;
	const int lq = warp & 3, cbase = (warp >> 2) * TC_COLS_T;
	const uint32_t trow = tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)cbase;
	while (cons.p < P1) {
		if (leader && ok) {
			if (!mbar_wait(fbars + 8 * slot, (fpar >> slot) & 1u)) { ok = false; atomicExch(err, 1); }
			fpar ^= 1u << slot;
			if (ok) {
				asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
				const uint32_t aS = sbase + (uint32_t)slot * TC_STAGE_BYTES, bS = aS + TC_A_BYTES;
#pragma unroll
				for (int kk = 0; kk < TC_KS / 16; ++kk)
					tc_mma(tmem, sw128_desc(aS + 32u * kk), sw128_desc(bS + 32u * kk), (fresh && kk == 0) ? 0u : 1u);
				tc_commit(mbars + 8 * slot);
				pending |= 1u << slot;
				// refill the slot the previous stage's MMAs read, once they are done
				const int prev = (slot + TC_NST - 1) % TC_NST;
				if (pending & (1u << prev)) {
					if (!mbar_wait(mbars + 8 * prev, (mpar >> prev) & 1u)) { ok = false; atomicExch(err, 1); }
					mpar ^= 1u << prev;
					pending &= ~(1u << prev);
				}
				if (ok) issue_stage(prod, prev);
			}
		}
		if (leader) advance(prod, Kp);
		fresh = false;
		const int p = cons.p;
		advance(cons, Kp);
		if (cons.p != p || cons.k0 == cons.kc0) {
			if (leader && ok && (pending & (1u << slot))) {
				if (!mbar_wait(mbars + 8 * slot, (mpar >> slot) & 1u)) { ok = false; atomicExch(err, 1); }
				mpar ^= 1u << slot;
				pending &= ~(1u << slot);
			}
			asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
			__syncthreads();	// the chunk's accumulator is complete
			asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
			const int d = c_pairs.s[p] + c_pairs.t[p];
			const int sh = d <= 3 ? BITS * (3 - d) : BITS * (NS - 1 - d);
			__syncwarp();	// tcgen05.ld is .sync.aligned: the warp converged
#pragma unroll
			for (int h = 0; h < TC_COLS_T / 32; ++h) {
				uint32_t v[32];
				tc_ld32(trow + 32u * h, v);
#pragma unroll
				for (int j = 0; j < 32; ++j) isum[32 * h + j] += (long long)__float2int_rn(__uint_as_float(v[j])) << sh;
			}
			asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
			__syncthreads();	// tensor memory read before the next chunk's first MMA overwrites it
			fresh = true;
		}
		slot = (slot + 1) % TC_NST;
	}
	// after a wait ran out: the MMAs still in flight finish (bounded waits) before tensor memory is freed
	if (leader)
		for (int q = 0; q < TC_NST; ++q)
			if (pending & (1u << q)) mbar_wait(mbars + 8 * q, (mpar >> q) & 1u);
	const long row = rowA0 + lq * 32 + (tid & 31);
	if (row < n) {
		const int ef_a = ea[row];
#pragma unroll
		for (int j = 0; j < TC_COLS_T; ++j) {
			const long col = rowB0 + cbase + j;
			if (col >= M) continue;
			if (HI) { hsum[row * M + col] = isum[j]; continue; }
			const long long hi = hsum[row * M + col], lo = isum[j];
			const int ef_b = eb[col];
			const int e = (ef_a ? ef_a - 1022 : -1022) + (ef_b ? ef_b - 1022 : -1022);
			const long long th = hi * 32 + (lo >> 30);
			const long long tl = lo & ((1ll << 30) - 1);
			const double v = fma((double)th, 0x1p-40, (double)tl * 0x1p-70);
			const long qq = col / jdiv, rr = col - qq * jdiv;
			out[qq * jouter + row * istride + rr] = scalbn(v, e);
		}
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
	__syncthreads();
	__syncwarp();
	if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
}

// ---------------------------------------------------------------- warp-specialised tcgen05 + TMA
// Warps 0-7 read the accumulator at the end of each exact-sum chunk (as k_oz_gemm_tc); warp 8 lane 0
// issues the TMA loads, warp 9 lane 0 the MMAs.  Their hand-offs are mbarriers: full[s] (TMA bytes
// landed: MMA may read stage s), empty[s] (the stage's MMAs done: TMA may refill it), and per
// accumulator (two in tensor memory, used by alternate chunks) tfull (the chunk's MMAs done: the
// accumulator may be read) and tempty (all 256 epilogue threads read it: it may be overwritten).  The
// MMA warp never waits for its own MMAs, and while the epilogue reads one accumulator the MMAs of the
// next chunk fill the other.  Every wait is bounded; a role whose wait runs
// out sets *err and stops, and the others then run out as well.
constexpr int WS_EPI = 256, WS_THREADS = WS_EPI + 64;
constexpr size_t WS_SMEM = (size_t)TC_STAGE_BYTES * TC_NST + 1024 + 16 * TC_NST + 48;

template <bool HI>
__global__ void __launch_bounds__(WS_THREADS, 1) k_oz_gemm_ws(const __grid_constant__ CUtensorMap mapA,
	const __grid_constant__ CUtensorMap mapB, const int* __restrict__ ea, const int* __restrict__ eb, long n, long M, long Kp,
	long long* __restrict__ hsum, double* __restrict__ out, long istride, long jdiv, long jouter, int* __restrict__ err)
{
	constexpr int P0 = HI ? 0 : LOPAIR, P1 = HI ? LOPAIR : NPAIR;
	extern __shared__ __align__(1024) unsigned char tsm[];
	const uint32_t sraw = smem_u32(tsm);
	const uint32_t sbase = (sraw + 1023u) & ~1023u;
	// two accumulators in tensor memory (columns 0-127 and 128-255), used by alternate chunks, each with
	// its own "full" and "empty" barrier
	const uint32_t fullb = sbase + TC_STAGE_BYTES * TC_NST, emptyb = fullb + 8 * TC_NST;
	const uint32_t tfull = emptyb + 8 * TC_NST, tempty = tfull + 16, tslot = tempty + 16;
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const long rowA0 = (long)blockIdx.y * TC_M, rowB0 = (long)blockIdx.x * TC_N;

	if (tid == 0) {
		for (int q = 0; q < TC_NST; ++q) { mbar_init(fullb + 8 * q, 1); mbar_init(emptyb + 8 * q, 1); }
		mbar_init(tfull, 1); mbar_init(tfull + 8, 1);
		mbar_init(tempty, WS_EPI); mbar_init(tempty + 8, WS_EPI);
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tslot), "r"(2 * TC_TMEM_COLS) : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
	uint32_t tmem;
	asm volatile("ld.shared.u32 %0, [%1];\n" : "=r"(tmem) : "r"(tslot) : "memory");

	if (warp == 8) {
		// ---- TMA producer
		if (lane == 0) {
			asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
			asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(&mapB)) : "memory");
			cursor c{P0, 0, 0};
			uint32_t epar = 0;
			for (long q = 0; c.p < P1; ++q) {
				const int slot = (int)(q % TC_NST);
				if (q >= TC_NST) {
					if (!mbar_wait(emptyb + 8 * slot, (epar >> slot) & 1u)) { atomicExch(err, 1); break; }
					epar ^= 1u << slot;
				}
				const uint32_t dA = sbase + (uint32_t)slot * TC_STAGE_BYTES;
				mbar_expect_tx(fullb + 8 * slot, TC_STAGE_BYTES);
				tma_load_2d(dA, &mapA, (int)c.k0, (int)(c_pairs.s[c.p] * n + rowA0), fullb + 8 * slot);
				tma_load_2d(dA + TC_A_BYTES, &mapB, (int)c.k0, (int)(c_pairs.t[c.p] * M + rowB0), fullb + 8 * slot);
				advance(c, Kp);
			}
		}
	} else if (warp == 9) {
		// ---- MMA issuer
		if (lane == 0) {
			cursor c{P0, 0, 0};
			uint32_t fpar = 0, tpar = 0;	// tpar bit b: parity of accumulator b's "empty" barrier
			bool fresh = true;
			long chunk = 0;
			for (long q = 0; c.p < P1; ++q) {
				const int slot = (int)(q % TC_NST), buf = (int)(chunk & 1);
				if (fresh && chunk >= 2) {	// the epilogue has read this accumulator's previous chunk
					if (!mbar_wait(tempty + 8 * buf, (tpar >> buf) & 1u)) { atomicExch(err, 1); break; }
					tpar ^= 1u << buf;
				}
				if (!mbar_wait(fullb + 8 * slot, (fpar >> slot) & 1u)) { atomicExch(err, 1); break; }
				fpar ^= 1u << slot;
				asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
				const uint32_t aS = sbase + (uint32_t)slot * TC_STAGE_BYTES, bS = aS + TC_A_BYTES;
				const uint32_t tacc = tmem + (uint32_t)(buf * TC_TMEM_COLS);
#pragma unroll
				for (int kk = 0; kk < TC_KS / 16; ++kk)
					tc_mma(tacc, sw128_desc(aS + 32u * kk), sw128_desc(bS + 32u * kk), (fresh && kk == 0) ? 0u : 1u);
				tc_commit(emptyb + 8 * slot);
				fresh = false;
				const int p = c.p;
				advance(c, Kp);
				if (c.p != p || c.k0 == c.kc0) {	// end of an exact-sum chunk
					tc_commit(tfull + 8 * buf);
					fresh = true;
					++chunk;
				}
			}
		}
	} else {
		// ---- epilogue warps 0-7: one accumulator read per chunk
		long long isum[TC_COLS_T];
#pragma unroll
		for (int j = 0; j < TC_COLS_T; ++j) isum[j] = 0;
		const int lq = warp & 3, cbase = (warp >> 2) * TC_COLS_T;
		const uint32_t trow = tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)cbase;
		cursor c{P0, 0, 0};
		uint32_t tpar = 0;	// bit b: parity of accumulator b's "full" barrier
		long chunk = 0;
		bool ok = true;
		while (c.p < P1) {
			const int p = c.p;
			advance(c, Kp);
			if (!(c.p != p || c.k0 == c.kc0)) continue;
			const int buf = (int)(chunk & 1);
			++chunk;
			if (ok && !mbar_wait(tfull + 8 * buf, (tpar >> buf) & 1u)) { ok = false; atomicExch(err, 1); }
			tpar ^= 1u << buf;
			if (!ok) break;
			asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
			__syncwarp();
			const int d = c_pairs.s[p] + c_pairs.t[p];
			const int sh = d <= 3 ? BITS * (3 - d) : BITS * (NS - 1 - d);
#pragma unroll
			for (int h = 0; h < TC_COLS_T / 32; ++h) {
				uint32_t v[32];
				tc_ld32(trow + (uint32_t)(buf * TC_TMEM_COLS) + 32u * h, v);
#pragma unroll
				for (int j = 0; j < 32; ++j) isum[32 * h + j] += (long long)__float2int_rn(__uint_as_float(v[j])) << sh;
			}
			asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
			asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(tempty + 8 * buf) : "memory");
		}
		const long row = rowA0 + lq * 32 + lane;
		if (ok && row < n) {
			const int ef_a = ea[row];
#pragma unroll
			for (int j = 0; j < TC_COLS_T; ++j) {
				const long col = rowB0 + cbase + j;
				if (col >= M) continue;
				if (HI) { hsum[row * M + col] = isum[j]; continue; }
				const long long hi = hsum[row * M + col], lo = isum[j];
				const int ef_b = eb[col];
				const int e = (ef_a ? ef_a - 1022 : -1022) + (ef_b ? ef_b - 1022 : -1022);
				const long long th = hi * 32 + (lo >> 30);
				const long long tl = lo & ((1ll << 30) - 1);
				const double v = fma((double)th, 0x1p-40, (double)tl * 0x1p-70);
				const long qq = col / jdiv, rr = col - qq * jdiv;
				out[qq * jouter + row * istride + rr] = scalbn(v, e);
			}
		}
	}
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
	__syncthreads();
	__syncwarp();
	if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(2 * TC_TMEM_COLS) : "memory");
}

} // namespace oz

size_t oz_digits_elems(long J, long K) { return (size_t)oz::NS * (size_t)J * (size_t)oz::pad16(K); }

// a wait of the tensor-core product that ran out (set by k_oz_gemm_tc, read and cleared by oz_check)
__device__ int g_oz_err;

// the product on the 5th-generation tensor cores (tcgen05, the default), or with the warp-level
// mma.sync kernel when QPC_OZ_TC=0 in the environment; both form the same exact sums
static bool oz_use_tc()
{
	const char* e = std::getenv("QPC_OZ_TC");
	return !(e && std::atoi(e) == 0);
}

// the operand loads of the tcgen05 path (QPC_OZ_TMA): 2 (default), TMA with producer, MMA and
// epilogue warps; 1, TMA from one thread that also issues the MMAs; 0, cp.async by all threads.
// Measured at n = K = 1880, M = 4000: 11.5, 6.9 and 8.3 TFLOP/s FP64-equivalent.
static int oz_tma_mode()
{
	const char* e = std::getenv("QPC_OZ_TMA");
	return e ? std::atoi(e) : 2;
}
static bool oz_use_tma() { return oz_use_tc() && oz_tma_mode() > 0; }

// tensor map of a digit array [rows][Kp] bf16: boxes of 64 k x box_rows rows, 128-byte swizzle (the
// layout the MMA descriptors read), zeros past the array.  The encoder comes from the driver through
// the runtime's entry-point query (no link against the driver library).
typedef CUresult (*encode_tiled_t)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
	const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static int digit_map(CUtensorMap* m, const __nv_bfloat16* D, long rows, long Kp, int box_rows)
{
	static encode_tiled_t enc = nullptr;
	if (!enc) {
		void* f = nullptr;
		cudaDriverEntryPointQueryResult q{};
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess || !f) {
			set_error("cuTensorMapEncodeTiled is not available");
			return QPC_ERR_CUDA;
		}
		enc = (encode_tiled_t)f;
	}
	const cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
	const cuuint64_t strides[1] = {(cuuint64_t)Kp * 2};
	const cuuint32_t box[2] = {(cuuint32_t)oz::TC_KS, (cuuint32_t)box_rows};
	const cuuint32_t estr[2] = {1, 1};
	if (enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)D, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
			CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
		set_error("cuTensorMapEncodeTiled failed (rows %ld, Kp %ld)", rows, Kp);
		return QPC_ERR_ARGS;
	}
	return QPC_OK;
}

int oz_check(cudaStream_t st)
{
	int* ep = nullptr;
	if (cudaGetSymbolAddress((void**)&ep, g_oz_err) != cudaSuccess) { set_error("oz_check: symbol"); return QPC_ERR_CUDA; }
	int h = 0;
	if (int rc = copy_to_host(&h, ep, sizeof(int), st)) return rc;
	if (h) {
		cudaMemsetAsync(ep, 0, sizeof(int), st);
		set_error("tensor-core product: an mbarrier wait ran out");
		return QPC_ERR_TIMEOUT;
	}
	return QPC_OK;
}

// exponent fields ef[J] and digit slices D[NS][J][pad16(K)] of an operand, enqueued on st
int oz_split(const oz::operand& o, long K, long J, int* ef, __nv_bfloat16* D, cudaStream_t st)
{
	if (K < 1 || J < 1) return QPC_OK;
	const long Kp = oz::pad16(K);
	if (cudaMemsetAsync(ef, 0, sizeof(int) * (size_t)J, st) != cudaSuccess) { set_error("oz_split: memset"); return QPC_ERR_CUDA; }
	const long gy = (K + oz::EXP_KR - 1) / oz::EXP_KR, gx = (J + 255) / 256;
	if (gy > 65535 || gx > 2147483647L) { set_error("oz_split: operand too large"); return QPC_ERR_ARGS; }
	oz::k_oz_exp<<<dim3((unsigned)gx, (unsigned)gy), 256, 0, st>>>(o, K, J, ef);
	const long sx = (J + 31) / 32, sy = (Kp + 31) / 32;
	if (sy > 65535) { set_error("oz_split: K too large"); return QPC_ERR_ARGS; }
	oz::k_oz_split<<<dim3((unsigned)sx, (unsigned)sy), dim3(32, 8), 0, st>>>(o, K, J, Kp, ef, D);
	return cudaGetLastError() == cudaSuccess ? QPC_OK : QPC_ERR_CUDA;
}

// out(i, j) = sum_k A(i, k) B(k, j), i < n, j < M, from the slices of A (rows) and B (columns);
// out(i, j) at out + (j / jdiv) * jouter + i * istride + j % jdiv
int oz_gemm(const __nv_bfloat16* Da, const int* ea, const __nv_bfloat16* Db, const int* eb, long n, long M, long K, double* out,
	long istride, long jdiv, long jouter, cudaStream_t st)
{
	if (n < 1 || M < 1) return QPC_OK;
	const long gx = (M + oz::TN - 1) / oz::TN, gy = (n + oz::TM - 1) / oz::TM;
	if (gy > 65535 || gx > 2147483647L) { set_error("oz_gemm: too large"); return QPC_ERR_ARGS; }
	static bool attr = false;	// the opt-in shared-memory size, once per process (all devices alike)
	if (!attr) {
		if (cudaFuncSetAttribute(oz::k_oz_gemm<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz::GEMM_SMEM) != cudaSuccess ||
			cudaFuncSetAttribute(oz::k_oz_gemm<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz::GEMM_SMEM) != cudaSuccess) {
			set_error("oz_gemm: shared-memory attribute");
			return QPC_ERR_CUDA;
		}
		attr = true;
	}
	// the exact sums of the digit levels 0..3, from the first launch to the second (stream-ordered)
	long long* hsum = nullptr;
	if (cudaMallocAsync((void**)&hsum, sizeof(long long) * (size_t)n * (size_t)M, st) != cudaSuccess) {
		set_error("oz_gemm: cudaMallocAsync of %ld x %ld level sums", n, M);
		return QPC_ERR_NOMEM;
	}
	if (oz_use_tma() && (long)oz::NS * n < (1L << 31) && (long)oz::NS * M < (1L << 31)) {
		static bool mattr = false;
		if (!mattr) {
			if (cudaFuncSetAttribute(oz::k_oz_gemm_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz::TMA_SMEM) != cudaSuccess ||
				cudaFuncSetAttribute(oz::k_oz_gemm_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz::TMA_SMEM) != cudaSuccess ||
				cudaFuncSetAttribute(oz::k_oz_gemm_ws<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz::WS_SMEM) != cudaSuccess ||
				cudaFuncSetAttribute(oz::k_oz_gemm_ws<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz::WS_SMEM) != cudaSuccess) {
				set_error("oz_gemm: shared-memory attribute (TMA)");
				cudaFreeAsync(hsum, st);
				return QPC_ERR_CUDA;
			}
			mattr = true;
		}
		CUtensorMap ma, mb;
		if (int rc = digit_map(&ma, Da, oz::NS * n, oz::pad16(K), oz::TC_M)) { cudaFreeAsync(hsum, st); return rc; }
		if (int rc = digit_map(&mb, Db, oz::NS * M, oz::pad16(K), oz::TC_N)) { cudaFreeAsync(hsum, st); return rc; }
		int* ep = nullptr;
		if (cudaGetSymbolAddress((void**)&ep, g_oz_err) != cudaSuccess) { set_error("oz_gemm: symbol"); cudaFreeAsync(hsum, st); return QPC_ERR_CUDA; }
		const dim3 tg((unsigned)((M + oz::TC_N - 1) / oz::TC_N), (unsigned)((n + oz::TC_M - 1) / oz::TC_M));
		if (oz_tma_mode() == 2) {
			oz::k_oz_gemm_ws<true><<<tg, oz::WS_THREADS, oz::WS_SMEM, st>>>(ma, mb, ea, eb, n, M, oz::pad16(K), hsum, out, istride, jdiv, jouter, ep);
			oz::k_oz_gemm_ws<false><<<tg, oz::WS_THREADS, oz::WS_SMEM, st>>>(ma, mb, ea, eb, n, M, oz::pad16(K), hsum, out, istride, jdiv, jouter, ep);
		} else {
			oz::k_oz_gemm_tma<true><<<tg, oz::TC_THREADS, oz::TMA_SMEM, st>>>(ma, mb, ea, eb, n, M, oz::pad16(K), hsum, out, istride, jdiv, jouter, ep);
			oz::k_oz_gemm_tma<false><<<tg, oz::TC_THREADS, oz::TMA_SMEM, st>>>(ma, mb, ea, eb, n, M, oz::pad16(K), hsum, out, istride, jdiv, jouter, ep);
		}
		cudaFreeAsync(hsum, st);
		return cudaGetLastError() == cudaSuccess ? QPC_OK : QPC_ERR_CUDA;
	}
	if (oz_use_tc() && n * oz::pad16(K) < (1L << 31) && M * oz::pad16(K) < (1L << 31)) {
		static bool tattr = false;
		if (!tattr) {
			if (cudaFuncSetAttribute(oz::k_oz_gemm_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz::TC_SMEM) != cudaSuccess ||
				cudaFuncSetAttribute(oz::k_oz_gemm_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz::TC_SMEM) != cudaSuccess) {
				set_error("oz_gemm: shared-memory attribute (tcgen05)");
				cudaFreeAsync(hsum, st);
				return QPC_ERR_CUDA;
			}
			tattr = true;
		}
		int* ep = nullptr;
		if (cudaGetSymbolAddress((void**)&ep, g_oz_err) != cudaSuccess) { set_error("oz_gemm: symbol"); cudaFreeAsync(hsum, st); return QPC_ERR_CUDA; }
		const dim3 tg((unsigned)((M + oz::TC_N - 1) / oz::TC_N), (unsigned)((n + oz::TC_M - 1) / oz::TC_M));
		oz::k_oz_gemm_tc<true><<<tg, oz::TC_THREADS, oz::TC_SMEM, st>>>(Da, ea, Db, eb, n, M, oz::pad16(K), hsum, out, istride, jdiv, jouter, ep);
		oz::k_oz_gemm_tc<false><<<tg, oz::TC_THREADS, oz::TC_SMEM, st>>>(Da, ea, Db, eb, n, M, oz::pad16(K), hsum, out, istride, jdiv, jouter, ep);
		cudaFreeAsync(hsum, st);
		return cudaGetLastError() == cudaSuccess ? QPC_OK : QPC_ERR_CUDA;
	}
	const dim3 grid((unsigned)gx, (unsigned)gy);
	oz::k_oz_gemm<true><<<grid, oz::THREADS, oz::GEMM_SMEM, st>>>(Da, ea, Db, eb, n, M, oz::pad16(K), hsum, out, istride, jdiv, jouter);
	oz::k_oz_gemm<false><<<grid, oz::THREADS, oz::GEMM_SMEM, st>>>(Da, ea, Db, eb, n, M, oz::pad16(K), hsum, out, istride, jdiv, jouter);
	cudaFreeAsync(hsum, st);
	return cudaGetLastError() == cudaSuccess ? QPC_OK : QPC_ERR_CUDA;
}

} // namespace qpc

using namespace qpc;

extern "C" int qpc_dgemm_slices(int64_t n, int64_t M, int64_t K, const double* A, int64_t lda, const double* B, int64_t ldb, double* C,
	int64_t ldc, float* ms)
{
	if (n < 1 || M < 1 || K < 1 || !A || !B || !C || lda < K || ldb < M || ldc < M) { set_error("qpc_dgemm_slices: bad arguments"); return QPC_ERR_ARGS; }
	int dev = 0;
	if (int rc = check_device(&dev)) return rc;
	cudaStream_t st = nullptr;
	QPC_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
	struct sguard { cudaStream_t s; ~sguard() { cudaStreamDestroy(s); } } sg{st};
	double *dA = nullptr, *dB = nullptr, *dC = nullptr;
	int *ea = nullptr, *eb = nullptr;
	__nv_bfloat16 *Da = nullptr, *Db = nullptr;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	auto release = [&]() {
		for (void* p : {(void*)dA, (void*)dB, (void*)dC, (void*)ea, (void*)eb, (void*)Da, (void*)Db}) if (p) cudaFreeAsync(p, st);
		if (e0) cudaEventDestroy(e0);
		if (e1) cudaEventDestroy(e1);
	};
	if (cudaMallocAsync((void**)&dA, sizeof(double) * (size_t)n * lda, st) != cudaSuccess ||
		cudaMallocAsync((void**)&dB, sizeof(double) * (size_t)K * ldb, st) != cudaSuccess ||
		cudaMallocAsync((void**)&dC, sizeof(double) * (size_t)n * ldc, st) != cudaSuccess ||
		cudaMallocAsync((void**)&ea, sizeof(int) * (size_t)n, st) != cudaSuccess ||
		cudaMallocAsync((void**)&eb, sizeof(int) * (size_t)M, st) != cudaSuccess ||
		cudaMallocAsync((void**)&Da, sizeof(__nv_bfloat16) * oz_digits_elems(n, K), st) != cudaSuccess ||
		cudaMallocAsync((void**)&Db, sizeof(__nv_bfloat16) * oz_digits_elems(M, K), st) != cudaSuccess ||
		cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
		set_error("qpc_dgemm_slices: device allocation failed");
		release();
		wait_on(st);
		return QPC_ERR_NOMEM;
	}
	int rc = QPC_OK;
	if (cudaMemcpyAsync(dA, A, sizeof(double) * (size_t)n * lda, cudaMemcpyHostToDevice, st) != cudaSuccess ||
		cudaMemcpyAsync(dB, B, sizeof(double) * (size_t)K * ldb, cudaMemcpyHostToDevice, st) != cudaSuccess) {
		set_error("qpc_dgemm_slices: upload failed");
		rc = QPC_ERR_CUDA;
	}
	// A(i, k) = A[i lda + k]: column j of the split is row i; B(k, j) = B[k ldb + j]
	if (!rc) rc = oz_split(oz::operand{dA, 1, lda, 0, n}, K, n, ea, Da, st);
	if (!rc) cudaEventRecord(e0, st);
	if (!rc) rc = oz_split(oz::operand{dB, ldb, 1, 0, M}, K, M, eb, Db, st);
	if (!rc) rc = oz_gemm(Da, ea, Db, eb, n, M, K, dC, ldc, M, 0, st);
	if (!rc) cudaEventRecord(e1, st);
	if (!rc) rc = wait_on(st);
	if (!rc) rc = oz_check(st);
	if (!rc && ms) cudaEventElapsedTime(ms, e0, e1);
	if (!rc) rc = copy_to_host(C, dC, sizeof(double) * (size_t)n * ldc, st);
	release();
	if (rc == QPC_OK) rc = wait_on(st);
	return rc;
}
