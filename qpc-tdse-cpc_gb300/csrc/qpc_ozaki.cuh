// FP64 matrix products on the bf16 tensor cores by exact integer slices (the Ozaki scheme:
// K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, "Error-free transformations of matrix multiplication
// by using fast routines of matrix multiplication and its applications", Numer. Algorithms 59, 2012;
// H. Ootomo, K. Ozaki, R. Yokota, "DGEMM on integer matrix multiplication unit", IJHPCA 2024).
//
// C = A B with A [n][K] and B [K][M] in FP64.  Every row i of A is written as
//     a_ik = 2^ea_i * sum_s alpha_s,ik 2^-7(s+1),   s = 0..NS-1 (NS = 9),
// alpha_s = the s-th group of 7 bits (most significant first) of trunc(|a| 2^(63 - ea_i)) with the
// sign of a, so |alpha| <= 127 is exact in bfloat16; every column j of B likewise with eb_j.  Then
//     c_ij = 2^(ea_i + eb_j) sum_{s+t<NS} 2^-7(s+t+2) sum_k alpha_s,ik beta_t,kj,
// and each inner sum over a chunk of KC = 1024 terms is an integer below 1024 * 127^2 < 2^24, so the
// tensor core's fp32 accumulation of bf16 products is exact.  The chunk sums are added as integers
// into two int64 accumulators per output (levels d = s + t <= 3, and 4..8, each shifted to a common
// scale) and rounded to FP64 once at the end.  The digits' truncation (2^-63 of each row's and
// column's power of two) and the pairs left out (s + t >= NS) keep the error near
// K 2^(ea_i + eb_j - 61), an order of magnitude below the rounding of an FP64 dot product.  The FP64
// pipe does no work in the inner loops (GB300 issues FP64 at a small fraction of the bf16 tensor
// rate): splitting uses integer operations on the FP64 bit patterns, and the products run on the
// tensor cores, as tcgen05.mma with the accumulator in tensor memory (the default) or as the
// warp-level mma.sync.m16n8k16 bf16 x bf16 -> fp32 (QPC_OZ_TC=0).
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <cstddef>

namespace qpc {
namespace oz {

constexpr int BITS = 7, NS = 9, KC = 1024;
constexpr int TM = 64, TN = 64, THREADS = 128;	// output tile, 4 warps of 32 x 32

// element (k, j) of an operand: p + (j / jdiv) * jouter + (j % jdiv) * jstride + k * kstride
struct operand {
	const double* p;
	long kstride, jstride, jouter;
	long jdiv;
};

constexpr int EXP_KR = 64;	// rows per block of the exponent pass

inline long pad16(long K) { return (K + 15) / 16 * 16; }

} // namespace oz

// host wrappers (qpc_ozaki.cu), enqueued on st without a wait
size_t oz_digits_elems(long J, long K);
int oz_split(const oz::operand& o, long K, long J, int* ef, __nv_bfloat16* D, cudaStream_t st);
// QPC_ERR_TIMEOUT (and clears it) when a wait of the tensor-core product ran out since the last check
int oz_check(cudaStream_t st);
int oz_gemm(const __nv_bfloat16* Da, const int* ea, const __nv_bfloat16* Db, const int* eb, long n, long M, long K, double* out,
	long istride, long jdiv, long jouter, cudaStream_t st);

} // namespace qpc
