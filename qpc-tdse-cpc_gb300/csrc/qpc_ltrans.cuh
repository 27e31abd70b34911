// The length-gauge l-space transform on the tcgen05 tensor cores (qpc_ltrans.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>

namespace qpc {

// half-width KB of the transform's block-diagonal product for n_l channels (16 for n_l <= 32, 24 for
// n_l <= 48), 0 when n_l is too large for it (the FP64 kernel k_transform serves those)
int ltrans_kb(int L);
// bytes of the digit planes of M eigensystems (both directions)
size_t ltrans_digit_bytes(int M, int KB);
// digit planes dig [M][2][8][2 KB][64] (bf16 bit patterns, 128-byte swizzled rows) and power-of-two
// exponents fex [M][2][2 KB] of the transform matrices built from Vh [M][npair+1][L] (host)
void ltrans_digits(const double* Vh, int M, int L, int npair, int KB, uint16_t* dig, int* fex);
// one transform (forward != 0: l basis -> eigen-basis slots, else back) of instances [b0, b0 + B) of an
// engine state [inst][m][r][l]; ntf != NULL skips instances without coupling work at loop step `step`
// (coupling_power).  A wait on the tensor core that runs out sets status |= stbit.  Enqueued on st;
// a launch error is left for the caller's cudaGetLastError.
int ltrans_launch(int KB, const double2* src, double2* dst, const uint16_t* dig, const int* fex, int N, int L, int M,
	int npair, int forward, const int64_t* ntf, long step, int b0, int B, int cmode, int* status, int stbit, cudaStream_t st);

} // namespace qpc
