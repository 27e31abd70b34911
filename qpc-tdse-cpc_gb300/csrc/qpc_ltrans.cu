// The l-space transform of the length-gauge coupling step (cn_transform_hl,
// spherical/propagator/cn_1e.hpp:101-147) on the tcgen05 tensor cores, at FP64 accuracy.
//
// Per position r of an (instance, m) block, the engine's even/odd transform (k_transform in
// qpc_engine.cu) is two small real products on the real and imaginary parts of the L channel values:
//     forward   E = Ve c_even,  O = Vo c_odd  ->  slots 2k = E_k + O_k, 2k+1 = conj(E_k - O_k), Z = E_np
//     backward  c_even = Ve^T (s, Z),  c_odd = Vo^T d
// (Ve: rows of the eigenvectors on even l, Vo: on odd l).  One tile is 64 positions x 2 parts = 128
// rows, multiplied by the block-diagonal matrix [Ve 0; 0 Vo] of half-width KB (K = N = 2 KB <= 48).
//
// Exact digits, as in the slice-product GEMM (qpc_ozaki.cuh) but with 8 digits of 8 bits: every row
// (the L values of one part at one position, both parities) is written under its power of two 2^e,
//     x = 2^(e - 63) Y,  Y = trunc(|x| 2^(63 - e)) < 2^63,  digit s = bits 56 - 8 s .. 63 - 8 s of Y,
// with the sign of x; each digit is at most 255 and exact in bfloat16.  The matrix's rows are split
// the same way (host, once).  The product keeps the digit pairs s + t <= 7 (36 pairs), one fp32
// accumulator in tensor memory per level d = s + t: a level sums at most 8 pairs x 24 nonzero terms x
// 255^2 < 2^24, so the tensor core's fp32 accumulation is exact.  The 8 levels are combined as
// integers, T = sum_d lev_d 2^(8 (7 - d)), rounded to FP64 once and scaled by 2^(e + f - 70):
// the result is the correctly rounded value of the truncated digit product, whose error is at most
// about 2^(e + f - 59) per term (the dropped pairs and the digits' truncation), 64 times below the
// rounding of an FP64 dot product.  The FP64 pipe, which GB300
// issues at a small fraction of its tensor rate, only rounds and combines the outputs.
//
// Pipeline of one block (128 threads, one per tile row): the thread splits its row into the 8 digit
// planes one plane at a time, into two plane buffers in shared memory (128-byte swizzled, K-major);
// thread 0 issues the plane's MMAs against the resident digit planes of the matrix and commits them
// to the buffer's mbarrier, so the next plane is written while the tensor core works.  After the last
// plane every thread reads its row's 8 accumulators (tcgen05.ld), rounds, combines and stores.  All
// mbarrier waits are bounded; a wait that runs out sets a status bit and the block stops issuing.
#include "qpc_internal.h"
#include "qpc_cuda_util.cuh"
#include "qpc_tcgen05.cuh"
#include "qpc_ltrans.cuh"
#include "qpc_chain.cuh"
#include <cuda_runtime.h>
#include <cstring>
#include <cmath>
#include <vector>
#include <algorithm>
#include <mutex>

namespace qpc {
namespace lt {

constexpr int NSL = 8, SBITS = 8;               // digits per value, bits per digit
constexpr int POS = 64, ROWS = 2 * POS, THREADS = ROWS;
constexpr int ACC_STRIDE = 64;                  // the accumulator of level d at tensor-memory column 64 d
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t PLANE_A = ROWS * 128;        // one digit plane of a tile: 128 rows x 64 bf16

template <int KB>
struct cfg {
	static constexpr int NT = 2 * KB;               // outputs = K extent: even block [0, KB), odd [KB, 2 KB)
	static constexpr int KSTEPS = NT / 16;
	static constexpr uint32_t PLANE_B = NT * 128;
	static constexpr uint32_t IDESC = tc::idesc_bf16(ROWS, NT);
	static constexpr uint32_t OFF_B = 2 * PLANE_A;                  // two A plane buffers, then the 8 B planes
	static constexpr uint32_t OFF_BAR = OFF_B + NSL * PLANE_B;      // 2 mbarriers, tensor-memory address
	static constexpr uint32_t OFF_FEX = OFF_BAR + 32;               // exponents of the matrix rows
	static constexpr size_t SMEM = OFF_FEX + 4 * NT + 1024;         // + alignment of the base to 1024 bytes
	static_assert(KB % 8 == 0 && NT % 16 == 0 && NT <= 64, "block width");
	static_assert(PLANE_B % 1024 == 0, "plane alignment");
	static_assert((NSL - 1) * ACC_STRIDE + NT <= (int)TMEM_COLS, "tensor memory");
};

// Y = trunc(|x| 2^(63 - e)) for a value with bit pattern b in a row with |x| < 2^e
__device__ __forceinline__ unsigned long long mant_scaled(unsigned long long b, int e)
{
	const int f = (int)((b >> 52) & 0x7ff);
	const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (f ? (1ull << 52) : 0ull);
	const int sh = (f ? f - 1023 : -1022) + 11 - e;
	return sh >= 0 ? (m << sh) : (sh > -64 ? (m >> -sh) : 0ull);
}

// bfloat16 bit pattern of the signed digit (y >> shift) & 255 (exact: at most 8 significant bits)
__device__ __forceinline__ uint32_t bf_digit(unsigned long long y, int shift, unsigned neg)
{
	const uint32_t d = (uint32_t)(y >> shift) & 255u;
	return (__float_as_uint((float)d) >> 16) | (neg << 15);
}

// 8 output columns col0 .. col0 + 7 of this thread's row: the 8 level accumulators combined exactly
// and rounded once; e = the row's exponent, fex = the matrix rows' exponents
__device__ __forceinline__ void round_cols(uint32_t tlane, int col0, int e, const int* fex, double (&out)[8])
{
	uint32_t v[NSL][8];
#pragma unroll
	for (int d = 0; d < NSL; ++d) tc::ld8(tlane + (uint32_t)(d * ACC_STRIDE + col0), v[d]);
	tc::wait_ld();
#pragma unroll
	for (int j = 0; j < 8; ++j) {
		long long hi = 0, lo = 0;
#pragma unroll
		for (int d = 0; d < 4; ++d) hi = hi * 256 + (long long)__float2int_rn(__uint_as_float(v[d][j]));
#pragma unroll
		for (int d = 4; d < NSL; ++d) lo = lo * 256 + (long long)__float2int_rn(__uint_as_float(v[d][j]));
		// T = hi 2^32 + lo = th 2^32 + tl with |th| < 2^50 and 0 <= tl < 2^32: both exact in FP64, one rounding
		const long long th = hi + (lo >> 32);
		const long long tl = lo & 0xFFFFFFFFll;
		const double x = fma((double)th, 0x1p32, (double)tl);
		out[j] = scalbn(x, e + fex[col0 + j] - 70);
	}
}

template <int KB>
__global__ void __launch_bounds__(THREADS, 1) k_ltrans(const double* __restrict__ src, double* __restrict__ dst,
	const uint4* __restrict__ bdig, const int* __restrict__ bexp, int N, int L, int M, int np, int forward,
	const int64_t* __restrict__ ntf, long step, int b0, long ntiles, int cmode, int* __restrict__ status, int stbit)
{
	using C = cfg<KB>;
	extern __shared__ __align__(1024) unsigned char lsm[];
	const uint32_t sraw = tc::smem_u32(lsm);
	const uint32_t pad = ((sraw + 1023u) & ~1023u) - sraw;
	unsigned char* base = lsm + pad;
	const uint32_t sA = sraw + pad, sB = sA + C::OFF_B, bar0 = sA + C::OFF_BAR, bar1 = bar0 + 8, tslot = bar0 + 16;
	int* fex = reinterpret_cast<int*>(base + C::OFF_FEX);
	const int tid = threadIdx.x, warp = tid >> 5;
	const int dir = forward ? 0 : 1;

	if (tid == 0) {
		tc::mbar_init(bar0, 1);
		tc::mbar_init(bar1, 1);
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tslot), "r"(TMEM_COLS) : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
	}
	tc::fence_before();
	__syncthreads();
	tc::fence_after();
	uint32_t tmem;
	asm volatile("ld.shared.u32 %0, [%1];\n" : "=r"(tmem) : "r"(tslot) : "memory");

	const int tpb = (N + POS - 1) / POS;
	const int q = tid >> 1, part = tid & 1;	// this thread's tile row: position q, real or imaginary part
	const uint32_t tlane = tmem + ((uint32_t)(warp * 32) << 16);
	const uint32_t rowA = (uint32_t)tid * 128u, swz = (uint32_t)(tid & 7);
	uint32_t ph[2] = {0u, 0u};	// completed waits per mbarrier (the next phase's parity = ph & 1)
	unsigned pend = 0;		// bit b: a commit to mbarrier b not waited for yet
	bool ok = true, stop = false;
	int loaded = -1;
	for (long t = blockIdx.x; t < ntiles && !stop; t += gridDim.x) {
		const long blk = t / tpb;
		const long im_inst = (long)b0 * M + blk;
		const int r0 = (int)(t - blk * tpb) * POS;
		const int m = (int)(im_inst % M);
		if (ntf && coupling_power(step, ntf[im_inst / M], cmode) == 0) continue;	// the same for the whole block
		const int nr = min(POS, N - r0);
		if (m != loaded) {
			__syncthreads();	// every thread is done with the previous exponents; no MMA is in flight
			const uint4* g = bdig + ((size_t)m * 2 + dir) * (NSL * C::PLANE_B / 16);
			uint4* s = reinterpret_cast<uint4*>(base + C::OFF_B);
			for (int i = tid; i < (int)(NSL * C::PLANE_B / 16); i += THREADS) s[i] = g[i];
			if (tid < C::NT) fex[tid] = bexp[((size_t)m * 2 + dir) * C::NT + tid];
			loaded = m;
		}
		const bool live = q < nr;
		const size_t rowoff = (((size_t)im_inst * N + r0 + q) * L) * 2 + part;
		// the row's values in the product's k order (even l, then odd l), zero past L
		unsigned long long y[C::NT];
		int fmax = 0;
#pragma unroll
		for (int k = 0; k < C::NT; ++k) {
			const int j = k < KB ? 2 * k : 2 * (k - KB) + 1;
			y[k] = (live && j < L) ? (unsigned long long)__double_as_longlong(__ldg(src + rowoff + 2 * j)) : 0ull;
			fmax = max(fmax, (int)((y[k] >> 52) & 0x7ff));
		}
		const int e = fmax ? fmax - 1022 : -1022;
		unsigned long long neg = 0;
#pragma unroll
		for (int k = 0; k < C::NT; ++k) {
			neg |= (y[k] >> 63) << k;
			y[k] = mant_scaled(y[k], e);
		}
#pragma unroll
		for (int s = 0; s < NSL; ++s) {
			const int b = s & 1;
			const uint32_t bar = b ? bar1 : bar0;
			if (pend & (1u << b)) {	// the MMAs that read this buffer two planes ago
				if (ok && !tc::mbar_wait(bar, ph[b] & 1u)) ok = false;
				++ph[b];
				pend &= ~(1u << b);
			}
			const uint32_t dA = sA + (uint32_t)b * PLANE_A + rowA;
			const int sh = SBITS * (NSL - 1 - s);
#pragma unroll
			for (int c = 0; c < C::NT / 8; ++c) {
				uint32_t w[4];
#pragma unroll
				for (int h = 0; h < 4; ++h) {
					const int k0 = 8 * c + 2 * h;
					w[h] = bf_digit(y[k0], sh, (unsigned)(neg >> k0) & 1u) |
						(bf_digit(y[k0 + 1], sh, (unsigned)(neg >> (k0 + 1)) & 1u) << 16);
				}
				asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" ::"r"(dA + ((((uint32_t)c) ^ swz) << 4)), "r"(w[0]),
					"r"(w[1]), "r"(w[2]), "r"(w[3]) : "memory");
			}
			tc::fence_async_smem();
			tc::fence_before();
			if (__syncthreads_or(ok ? 0 : 1)) { stop = true; break; }	// the block stops together
			tc::fence_after();
			if (tid == 0) {
				const uint32_t aP = sA + (uint32_t)b * PLANE_A;
				for (int u = 0; u + s < NSL; ++u) {
					const uint32_t acc = tmem + (uint32_t)((s + u) * ACC_STRIDE);
					const uint32_t bP = sB + (uint32_t)u * C::PLANE_B;
#pragma unroll
					for (int kk = 0; kk < C::KSTEPS; ++kk)
						tc::mma_bf16(acc, tc::sw128_desc(aP + 32u * kk), tc::sw128_desc(bP + 32u * kk), C::IDESC,
							(s > 0 || kk > 0) ? 1u : 0u);
				}
				tc::commit(bar);
			}
			pend |= 1u << b;
		}
		if (stop) break;
		for (int b = 0; b < 2; ++b)
			if (pend & (1u << b)) {
				if (ok && !tc::mbar_wait(b ? bar1 : bar0, ph[b] & 1u)) ok = false;
				++ph[b];
				pend &= ~(1u << b);
			}
		if (__syncthreads_or(ok ? 0 : 1)) break;
		tc::fence_after();
		double* orow = dst + rowoff;
#pragma unroll
		for (int c = 0; c < KB / 8; ++c) {
			double ev[8], ov[8];
			round_cols(tlane, 8 * c, e, fex, ev);
			round_cols(tlane, KB + 8 * c, e, fex, ov);
			if (live) {
#pragma unroll
				for (int j = 0; j < 8; ++j) {
					const int k = 8 * c + j;
					if (forward) {
						if (k < np) {
							orow[4 * k] = ev[j] + ov[j];
							orow[4 * k + 2] = part ? ov[j] - ev[j] : ev[j] - ov[j];
						} else if (k == np && (L & 1)) {
							orow[4 * k] = ev[j];
						}
					} else {
						if (2 * k < L) orow[4 * k] = ev[j];
						if (2 * k + 1 < L) orow[4 * k + 2] = ov[j];
					}
				}
			}
		}
		tc::fence_before();
	}
	// commits left after a wait ran out: wait for them (bounded) before the tensor memory is freed
	for (int b = 0; b < 2; ++b)
		if (pend & (1u << b)) tc::mbar_wait(b ? bar1 : bar0, ph[b] & 1u);
	if (!ok) atomicOr(status, stbit);
	tc::fence_before();
	__syncthreads();
	tc::fence_after();
	if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

} // namespace lt

int ltrans_kb(int L)
{
	if (L < 1) return 0;
	return L <= 32 ? 16 : (L <= 48 ? 24 : 0);
}

size_t ltrans_digit_bytes(int M, int KB) { return (size_t)M * 2 * lt::NSL * (2 * KB) * 128; }

// The host split of the transform matrices, the same digits as the kernel's rows (mant_scaled).
void ltrans_digits(const double* Vh, int M, int L, int np, int KB, uint16_t* dig, int* fex)
{
	const int NT = 2 * KB, ne = (L + 1) / 2, no = L / 2;
	std::vector<double> Bm((size_t)NT * NT);
	std::memset(dig, 0, ltrans_digit_bytes(M, KB));
	for (int m = 0; m < M; ++m)
		for (int dir = 0; dir < 2; ++dir) {
			std::fill(Bm.begin(), Bm.end(), 0.0);
			const double* V = Vh + (size_t)m * (np + 1) * L;
			// row n of the product's matrix = output n; forward: eigenvector n on even (odd) l;
			// backward: component 2n (2n + 1) of every eigenvector
			for (int n = 0; n < ne; ++n)
				for (int k = 0; k < ne; ++k) Bm[(size_t)n * NT + k] = dir == 0 ? V[(size_t)n * L + 2 * k] : V[(size_t)k * L + 2 * n];
			for (int n = 0; n < no; ++n)
				for (int k = 0; k < no; ++k)
					Bm[(size_t)(KB + n) * NT + KB + k] = dir == 0 ? V[(size_t)n * L + 2 * k + 1] : V[(size_t)k * L + 2 * n + 1];
			uint16_t* D = dig + ((size_t)m * 2 + dir) * lt::NSL * NT * 64;
			int* fx = fex + ((size_t)m * 2 + dir) * NT;
			for (int n = 0; n < NT; ++n) {
				int fm = 0;
				for (int k = 0; k < NT; ++k) {
					uint64_t b;
					std::memcpy(&b, &Bm[(size_t)n * NT + k], 8);
					fm = std::max(fm, (int)((b >> 52) & 0x7ff));
				}
				const int e = fm ? fm - 1022 : -1022;
				fx[n] = e;
				for (int k = 0; k < NT; ++k) {
					uint64_t b;
					std::memcpy(&b, &Bm[(size_t)n * NT + k], 8);
					const int f = (int)((b >> 52) & 0x7ff);
					const uint64_t mm = (b & 0xFFFFFFFFFFFFFull) | (f ? (1ull << 52) : 0ull);
					const int sh = (f ? f - 1023 : -1022) + 11 - e;
					const uint64_t y = sh >= 0 ? (mm << sh) : (sh > -64 ? (mm >> -sh) : 0ull);
					const size_t at = (size_t)n * 64 + (size_t)((((k >> 3) ^ (n & 7)) << 3) + (k & 7));
					for (int s = 0; s < lt::NSL; ++s) {
						const uint32_t d = (uint32_t)(y >> (lt::SBITS * (lt::NSL - 1 - s))) & 255u;
						const float fd = (float)d;
						uint32_t fb;
						std::memcpy(&fb, &fd, 4);
						D[(size_t)s * NT * 64 + at] = (uint16_t)((fb >> 16) | ((b >> 63) ? 0x8000u : 0u));
					}
				}
			}
		}
}

int ltrans_launch(int KB, const double2* src, double2* dst, const uint16_t* dig, const int* fex, int N, int L, int M,
	int np, int forward, const int64_t* ntf, long step, int b0, int B, int cmode, int* status, int stbit, cudaStream_t st)
{
	const long ntiles = (long)B * M * ((N + lt::POS - 1) / lt::POS);
	if (ntiles <= 0) return QPC_OK;
	int dev = 0;
	QPC_CUDA(cudaGetDevice(&dev));
	static std::mutex mu;
	static int nsm[64] = {0};
	static bool attr[64][2] = {};
	const int di = dev & 63, ki = KB == 16 ? 0 : 1;
	{
		std::lock_guard<std::mutex> lk(mu);
		if (!nsm[di]) QPC_CUDA(cudaDeviceGetAttribute(&nsm[di], cudaDevAttrMultiProcessorCount, dev));
		if (!attr[di][ki]) {
			if (KB == 16)
				QPC_CUDA(cudaFuncSetAttribute(lt::k_ltrans<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lt::cfg<16>::SMEM));
			else
				QPC_CUDA(cudaFuncSetAttribute(lt::k_ltrans<24>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lt::cfg<24>::SMEM));
			attr[di][ki] = true;
		}
	}
	const unsigned grid = (unsigned)std::min<long>(ntiles, nsm[di]);
	const double* s = reinterpret_cast<const double*>(src);
	double* d = reinterpret_cast<double*>(dst);
	const uint4* g = reinterpret_cast<const uint4*>(dig);
	if (KB == 16)
		lt::k_ltrans<16><<<grid, lt::THREADS, lt::cfg<16>::SMEM, st>>>(s, d, g, fex, N, L, M, np, forward, ntf, step, b0, ntiles,
			cmode, status, stbit);
	else if (KB == 24)
		lt::k_ltrans<24><<<grid, lt::THREADS, lt::cfg<24>::SMEM, st>>>(s, d, g, fex, N, L, M, np, forward, ntf, step, b0, ntiles,
			cmode, status, stbit);
	else {
		set_error("l-space transform: no tensor-core form for n_l = %d", L);
		return QPC_ERR_ARGS;
	}
	return QPC_OK;	// a launch error stays for the caller's cudaGetLastError
}

} // namespace qpc

// ---------------------------------------------------------------- C ABI
extern "C" int qpc_lspace_transform(int64_t n_pos, int n_l, const double* V, int forward, const double* in, double* out)
{
	using namespace qpc;
	const int KB = ltrans_kb(n_l);
	if (n_pos < 1 || !V || !in || !out || !KB) {
		set_error("qpc_lspace_transform: bad arguments (n_pos >= 1, 1 <= n_l <= 48, non-NULL buffers)");
		return QPC_ERR_ARGS;
	}
	if (n_pos > (int64_t)1 << 30) { set_error("qpc_lspace_transform: n_pos too large"); return QPC_ERR_ARGS; }
	int dev = 0;
	if (int rc = check_device(&dev)) return rc;
	const int np = n_l / 2;
	std::vector<uint16_t> dig(ltrans_digit_bytes(1, KB) / 2);
	std::vector<int> fex(2 * 2 * KB);
	ltrans_digits(V, 1, n_l, np, KB, dig.data(), fex.data());
	cudaStream_t st = nullptr;
	QPC_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
	struct sguard { cudaStream_t s; ~sguard() { cudaStreamDestroy(s); } } sg{st};
	const size_t nv = (size_t)n_pos * n_l * 2;
	double *din = nullptr, *dout = nullptr;
	uint16_t* ddig = nullptr;
	int *dfex = nullptr, *dstat = nullptr;
	auto release = [&]() {
		for (void* p : {(void*)din, (void*)dout, (void*)ddig, (void*)dfex, (void*)dstat}) if (p) cudaFreeAsync(p, st);
	};
	if (cudaMallocAsync((void**)&din, sizeof(double) * nv, st) != cudaSuccess ||
		cudaMallocAsync((void**)&dout, sizeof(double) * nv, st) != cudaSuccess ||
		cudaMallocAsync((void**)&ddig, sizeof(uint16_t) * dig.size(), st) != cudaSuccess ||
		cudaMallocAsync((void**)&dfex, sizeof(int) * fex.size(), st) != cudaSuccess ||
		cudaMallocAsync((void**)&dstat, sizeof(int), st) != cudaSuccess) {
		set_error("qpc_lspace_transform: device allocation failed");
		release();
		wait_on(st);
		return QPC_ERR_NOMEM;
	}
	int rc = QPC_OK;
	if (cudaMemcpyAsync(din, in, sizeof(double) * nv, cudaMemcpyHostToDevice, st) != cudaSuccess ||
		cudaMemcpyAsync(ddig, dig.data(), sizeof(uint16_t) * dig.size(), cudaMemcpyHostToDevice, st) != cudaSuccess ||
		cudaMemcpyAsync(dfex, fex.data(), sizeof(int) * fex.size(), cudaMemcpyHostToDevice, st) != cudaSuccess ||
		cudaMemsetAsync(dstat, 0, sizeof(int), st) != cudaSuccess ||
		cudaMemsetAsync(dout, 0, sizeof(double) * nv, st) != cudaSuccess) {
		set_error("qpc_lspace_transform: upload failed");
		rc = QPC_ERR_CUDA;
	}
	if (!rc)
		rc = ltrans_launch(KB, reinterpret_cast<const double2*>(din), reinterpret_cast<double2*>(dout), ddig, dfex, (int)n_pos, n_l, 1,
			np, forward, nullptr, 0, 0, 1, 0, dstat, 1, st);
	if (!rc && cudaGetLastError() != cudaSuccess) { set_error("qpc_lspace_transform: launch failed"); rc = QPC_ERR_CUDA; }
	int stat = 0;
	if (!rc) rc = copy_to_host(&stat, dstat, sizeof(int), st);
	if (!rc && stat) { set_error("qpc_lspace_transform: a tensor-core wait ran out"); rc = QPC_ERR_TIMEOUT; }
	if (!rc) rc = copy_to_host(out, dout, sizeof(double) * nv, st);
	release();
	if (rc == QPC_OK) rc = wait_on(st);
	return rc;
}
