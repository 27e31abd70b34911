// FP64 GEMM kernels for the dense (m,l) transforms of the velocity-gauge step
// (cn_transform_hm::construct/eliminate, spherical/propagator/cn_1e.hpp:151-293).
//
//   C[b] = op(A) B[b],  b < batch
//
// A is one real n x n matrix shared by the batch (row-major, leading dimension n), op(A) is A
// or A^T.  B[b] and C[b] are K x X row-major with leading dimension ld and batch stride sb: the
// rows [channel][2 N_r reals] of one m-parity set of one wavefunction's state (a real transform
// of a complex state), K = M = n channels.
//
// GB300 mapping.  FP64 runs at ~1.2 TFLOP/s (one warp-wide DFMA per ~64 cycles per SM
// sub-partition), HBM at ~6.7 TB/s: a transform with n ~ 3700 does ~n/2 flops per byte it
// moves, far above the machine balance, so the kernels are FP64-pipe-bound and the design
// goal is that nearly every issued FP64 instruction is a DFMA of the product.  Each block
// computes a 64 x 64 tile of C with 256 threads, 4 x 4 outputs per thread in registers;
// K advances in slices of 16 staged in shared memory (double-buffered, one barrier per
// slice), the next slice's global values prefetched into registers while the current one
// is consumed.  The tensor-core FP64 path (DMMA) shares the FP64 pipe on this part and
// measured slower than DFMA, so the product is plain DFMA; the transpose is folded into the
// A-tile load.
#pragma once
#include <cuda_runtime.h>

namespace qpc {
namespace gemm {

constexpr int BM = 64, BX = 64, BK = 16, THREADS = 256;

// real: C[b][i][x] = sum_j op(A)(i, j) B[b][j][x]; TRANS: op(A)(i, j) = A[j][i]
template <bool TRANS>
__global__ void __launch_bounds__(THREADS, 2) k_dgemm(const double* __restrict__ A, int n, const double* __restrict__ B,
	double* __restrict__ C, long ld, long sb, int X)
{
	__shared__ __align__(16) double As[2][BK][BM];
	__shared__ __align__(16) double Bs[2][BK][BX];
	const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
	const int i0 = blockIdx.y * BM, x0 = blockIdx.x * BX;
	const double* Bb = B + (long)blockIdx.z * sb;
	double* Cb = C + (long)blockIdx.z * sb;
	// global -> register assignment of one K slice: A 64 x 16 and B 16 x 64, 4 values each
	double ra[4], rb[4];
	auto load = [&](int k0) {
#pragma unroll
		for (int q = 0; q < 4; ++q) {
			const int e = tid + q * THREADS;	// 0..1023
			int ii, kk;
			if (TRANS) { kk = e >> 6; ii = e & 63; }	// A[k0+kk][i0+ii]: contiguous in i
			else { ii = e >> 4; kk = e & 15; }		// A[i0+ii][k0+kk]: contiguous in k
			const int gi = i0 + ii, gk = k0 + kk;
			ra[q] = (gi < n && gk < n) ? (TRANS ? A[(long)gk * n + gi] : A[(long)gi * n + gk]) : 0.0;
			const int bk = e >> 6, bx = e & 63;
			const int gb = k0 + bk, gx = x0 + bx;
			rb[q] = (gb < n && gx < X) ? Bb[(long)gb * ld + gx] : 0.0;
		}
	};
	auto store = [&](int buf) {
#pragma unroll
		for (int q = 0; q < 4; ++q) {
			const int e = tid + q * THREADS;
			int ii, kk;
			if (TRANS) { kk = e >> 6; ii = e & 63; }
			else { ii = e >> 4; kk = e & 15; }
			As[buf][kk][ii] = ra[q];
			Bs[buf][e >> 6][e & 63] = rb[q];
		}
	};
	double acc[4][4];
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int c = 0; c < 4; ++c) acc[a][c] = 0.0;
	const int nk = (n + BK - 1) / BK;
	load(0);
	store(0);
	__syncthreads();
	for (int t = 0; t < nk; ++t) {
		const int buf = t & 1;
		if (t + 1 < nk) load((t + 1) * BK);
#pragma unroll
		for (int k = 0; k < BK; ++k) {
			// rows ty + 16 a, columns 4 tx .. 4 tx + 3
			double av[4], bv[4];
#pragma unroll
			for (int a = 0; a < 4; ++a) av[a] = As[buf][k][ty + 16 * a];
			const double2 b01 = *reinterpret_cast<const double2*>(&Bs[buf][k][4 * tx]);
			const double2 b23 = *reinterpret_cast<const double2*>(&Bs[buf][k][4 * tx + 2]);
			bv[0] = b01.x; bv[1] = b01.y; bv[2] = b23.x; bv[3] = b23.y;
#pragma unroll
			for (int a = 0; a < 4; ++a)
#pragma unroll
				for (int c = 0; c < 4; ++c) acc[a][c] = fma(av[a], bv[c], acc[a][c]);
		}
		if (t + 1 < nk) store(buf ^ 1);
		__syncthreads();
	}
#pragma unroll
	for (int a = 0; a < 4; ++a) {
		const int gi = i0 + ty + 16 * a;
		if (gi >= n) continue;
#pragma unroll
		for (int c = 0; c < 4; ++c) {
			const int gx = x0 + 4 * tx + c;
			if (gx < X) Cb[(long)gi * ld + gx] = acc[a][c];
		}
	}
}

// grid of one launch: X columns, n rows, batch matrices (batch <= 65535)
inline dim3 grid_for(int X, int n, int batch)
{
	return dim3((unsigned)((X + BX - 1) / BX), (unsigned)((n + BM - 1) / BM), (unsigned)batch);
}

} // namespace gemm
} // namespace qpc
