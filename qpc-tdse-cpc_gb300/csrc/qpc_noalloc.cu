// Field-free Crank-Nicolson step for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a host framework that
// owns every device allocation through its own pool (and accounts for it),
// code that runs while a CUDA stream is being captured into a graph, or an
// embedding that has a fixed device-memory budget set up front.  They pass
// their own device buffers for the inputs and the result; the entry point
// below then needs no allocation at all.  Its scratch (the wavefunctions in
// the engine's r-major layout and the chain work vectors) lives in the
// file-scope array g_noalloc_scratch, which every GPU that loads this
// library holds until the process exits.
//
// The step is the one cn_hc_propagate0 performs (spherical/propagator/
// propagate.hpp:311-331), with the same chain kernel the handle-based engine
// uses (qpc_chain.cuh), unchanged.
#include "qpc_internal.h"
#include <cuda_runtime.h>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include "qpc_chain.cuh"

namespace qpc {

// two halves of QPC_NOALLOC_MAX_ELEMS complex128 values each: the state in
// engine layout, then the work vectors (2 x 16 MiB = 32 MiB per device)
static __device__ __align__(256) double2 g_noalloc_scratch[2 * QPC_NOALLOC_MAX_ELEMS];

namespace {

// device address of the scratch per device ordinal, looked up in the CUDA runtime's
// primary context of that device (the context cudaSetDevice makes current)
constexpr int kMaxDevices = 64;
double2* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

// reference layout [blk][l][r] <-> engine layout [blk][r][l]
__global__ void k_noalloc_to_rmajor(const double2* __restrict__ src, double2* __restrict__ dst, int N, int L, long nblk)
{
	long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= nblk * (long)N * L) return;
	long b = t / ((long)N * L);
	int rem = (int)(t % ((long)N * L));
	int r = rem / L, l = rem % L;
	dst[t] = src[b * (long)N * L + (long)l * N + r];
}
__global__ void k_noalloc_to_lmajor(const double2* __restrict__ src, double2* __restrict__ dst, int N, int L, long nblk)
{
	long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= nblk * (long)N * L) return;
	long b = t / ((long)N * L);
	int rem = (int)(t % ((long)N * L));
	int l = rem / N, r = rem % N;
	dst[t] = src[b * (long)N * L + (long)r * L + l];
}

__global__ void k_noalloc_fill(int64_t* __restrict__ t, long n, int64_t v)
{
	long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) t[i] = v;
}

template <int P, int G>
cudaError_t launch_ff(cudaStream_t st, double2* X, double2* W, const double2* ffac, const double* S, const int64_t* nta,
	int B, int M, int m0, int N, int L, size_t smem)
{
	using C = chain_cfg<P, G, false>;
	cudaError_t e = cudaFuncSetAttribute(k_chain<P, G, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	long nch = (long)B * M * L;
	long nwarps = (nch + C::CPW - 1) / C::CPW;
	unsigned grid = (unsigned)((nwarps + 3) / 4);
	// field-free chains run while step < nt_total[inst]: step 0 and a table of ones
	k_chain<P, G, false><<<grid, 128, smem, st>>>(X, W, ffac, S, nta, 0, 0, B, M, m0, N, L, L / 2, 0, nch);
	return cudaGetLastError();
}

template <int P>
cudaError_t dispatch(int many, cudaStream_t st, double2* X, double2* W, const double2* ffac, const double* S, const int64_t* nta,
	int B, int M, int m0, int N, int L, size_t smem)
{
	// many chains: one lane per real/imaginary part; few chains: P lanes per part
	if (many) return launch_ff<P, 1>(st, X, W, ffac, S, nta, B, M, m0, N, L, smem);
	return launch_ff<P, P>(st, X, W, ffac, S, nta, B, M, m0, N, L, smem);
}

} // namespace
} // namespace qpc

using namespace qpc;

extern "C" int qpc_fieldfree_noalloc(const qpc_dims* dims, const double* S, const double* ffac, double* coef, void* stream)
{
	if (!dims || !S || !ffac || !coef) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	const qpc_dims d = *dims;
	if (d.p < 3 || d.p > QPC_MAX_RANK || d.n_r < 2 * d.p + 2 || d.n_l < 1 || d.n_m < 1 || d.n_inst < 1) {
		set_error("bad dims n_r=%d p=%d n_l=%d n_m=%d n_inst=%d", d.n_r, d.p, d.n_l, d.n_m, d.n_inst);
		return QPC_ERR_ARGS;
	}
	const long elems = (long)d.n_inst * d.n_m * d.n_l * d.n_r;
	// the last QPC_NOALLOC_MAX_ELEMS/... entries of the work half hold the per-instance
	// step table (one int64 per instance, i.e. one double2 per two instances)
	const long table = (d.n_inst + 1) / 2;
	if (elems + table > QPC_NOALLOC_MAX_ELEMS) {
		set_error("qpc_fieldfree_noalloc: %ld complex values exceed the fixed scratch of %ld (n_inst*n_m*n_l*n_r + n_inst/2 must be <= %ld)",
			elems + table, (long)QPC_NOALLOC_MAX_ELEMS, (long)QPC_NOALLOC_MAX_ELEMS);
		return QPC_ERR_ARGS;
	}
	const size_t smem = sizeof(double) * (size_t)d.n_r * (d.p + 1);
	if (smem > 200 * 1024) { set_error("n_r=%d too large for the shared-memory S band", d.n_r); return QPC_ERR_ARGS; }
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) { set_error("cudaGetDevice: %s", cudaGetErrorString(e)); return QPC_ERR_NODEVICE; }
	if (dev < 0 || dev >= kMaxDevices) { set_error("device ordinal %d out of range", dev); return QPC_ERR_NODEVICE; }
	double2* base;
	{
		// set-up, once per device, with that device current: the device address of the scratch
		std::lock_guard<std::mutex> lk(g_scratch_mu);
		if (!g_scratch_ptr[dev]) {
			void* p = nullptr;
			e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
			if (e != cudaSuccess || !p) { set_error("cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e)); return QPC_ERR_CUDA; }
			g_scratch_ptr[dev] = static_cast<double2*>(p);
		}
		base = g_scratch_ptr[dev];
	}
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	double2* X = base;
	double2* W = base + QPC_NOALLOC_MAX_ELEMS;
	int64_t* nta = reinterpret_cast<int64_t*>(W + QPC_NOALLOC_MAX_ELEMS - table);
	const long nblk = (long)d.n_inst * d.n_m;
	// every instance takes the step: nt_total = 1 > step 0 (rewritten by every call;
	// the scratch keeps whatever the previous call left)
	k_noalloc_fill<<<(unsigned)((d.n_inst + 255) / 256), 256, 0, st>>>(nta, d.n_inst, 1);
	unsigned g = (unsigned)((elems + 255) / 256);
	k_noalloc_to_rmajor<<<g, 256, 0, st>>>(reinterpret_cast<const double2*>(coef), X, d.n_r, d.n_l, nblk);
	int many = (long)d.n_inst * d.n_m * d.n_l >= 4096;
	switch (d.p) {
	case 3: e = dispatch<3>(many, st, X, W, reinterpret_cast<const double2*>(ffac), S, nta, d.n_inst, d.n_m, d.m0, d.n_r, d.n_l, smem); break;
	case 4: e = dispatch<4>(many, st, X, W, reinterpret_cast<const double2*>(ffac), S, nta, d.n_inst, d.n_m, d.m0, d.n_r, d.n_l, smem); break;
	case 5: e = dispatch<5>(many, st, X, W, reinterpret_cast<const double2*>(ffac), S, nta, d.n_inst, d.n_m, d.m0, d.n_r, d.n_l, smem); break;
	case 6: e = dispatch<6>(many, st, X, W, reinterpret_cast<const double2*>(ffac), S, nta, d.n_inst, d.n_m, d.m0, d.n_r, d.n_l, smem); break;
	case 7: e = dispatch<7>(many, st, X, W, reinterpret_cast<const double2*>(ffac), S, nta, d.n_inst, d.n_m, d.m0, d.n_r, d.n_l, smem); break;
	default: e = dispatch<8>(many, st, X, W, reinterpret_cast<const double2*>(ffac), S, nta, d.n_inst, d.n_m, d.m0, d.n_r, d.n_l, smem); break;
	}
	if (e != cudaSuccess) { set_error("field-free chain launch: %s", cudaGetErrorString(e)); return QPC_ERR_CUDA; }
	k_noalloc_to_lmajor<<<g, 256, 0, st>>>(X, reinterpret_cast<double2*>(coef), d.n_r, d.n_l, nblk);
	e = cudaGetLastError();
	if (e != cudaSuccess) { set_error("layout launch: %s", cudaGetErrorString(e)); return QPC_ERR_CUDA; }
	return QPC_OK;
}
