// Host side of the slice-product FP64 GEMM (qpc_ozaki.cuh): splitting an operand into its digit
// slices, the product, and qpc_dgemm_slices, the C ABI form on host buffers.
#include "qpc_internal.h"
#include "qpc_cuda_util.cuh"
#include "qpc_ozaki.cuh"
#include <cuda_runtime.h>
#include <vector>

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

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

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

} // namespace oz

size_t oz_digits_elems(long J, long K) { return (size_t)oz::NS * (size_t)J * (size_t)oz::pad16(K); }

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
	if (!rc && ms) cudaEventElapsedTime(ms, e0, e1);
	if (!rc) rc = copy_to_host(C, dC, sizeof(double) * (size_t)n * ldc, st);
	release();
	if (rc == QPC_OK) rc = wait_on(st);
	return rc;
}
