// Harmonic spectra of many wavefunctions on the GPU: the spectrum reduction of a batched run.
//
// The quantity is the one qpc_hhg_spectrum computes on the host for one dipole list
// (analysis/plot_hhs.m restated): d(t_j) = -z(t_j) times the sin^2 window on (tmin, tmax),
// D(w_k) = DFT(d)_k dt / (2 pi) at w_k = 2 pi k / (n dt), S(w_k) = 4 pi^2 w^{+-2} |D|^2 / c^2.
// A batch of wavefunctions needs only the frequencies up to some harmonic order, not all n/2 of
// an FFT, so each block evaluates KPB frequencies of one list directly: every thread takes a
// strided share of the samples and the exact twiddles e^{-2 pi i (k j mod n) / n} come from a
// per-list table (index advanced by integer adds, no trigonometry in the sum); the block then
// reduces its partial sums in a fixed order, so results are deterministic.  FP64 throughout.
#include "qpc_internal.h"
#include "qpc_cuda_util.cuh"
#include <cuda_runtime.h>
#include <cmath>
#include <vector>

namespace qpc {
namespace {

constexpr int HT = 256, KPB = 8;

// w[inst][m] = e^{-2 pi i m / n[inst]}, m < n[inst]
__global__ void k_hhg_twiddle(const long long* __restrict__ n, long ldw, double2* __restrict__ w)
{
	const int inst = blockIdx.y;
	const long m = (long)blockIdx.x * blockDim.x + threadIdx.x;
	const long nn = n[inst];
	if (m >= nn) return;
	double s, c;
	sincospi(-2.0 * (double)m / (double)nn, &s, &c);
	w[(long)inst * ldw + m] = make_double2(c, s);
}

__global__ void __launch_bounds__(HT) k_hhg_dft(const double* __restrict__ x, long ldx, const double2* __restrict__ w, long ldw,
	const long long* __restrict__ n, long kmax, double dt, int type, double* __restrict__ spec)
{
	__shared__ double red[2][KPB][HT];
	const int inst = blockIdx.y, tid = threadIdx.x;
	const long k0 = (long)blockIdx.x * KPB;
	const long nn = n[inst];
	const double* xi = x + (long)inst * ldx;
	const double2* wi = w + (long)inst * ldw;
	double ar[KPB], ai[KPB];
	long idx[KPB], stp[KPB];
#pragma unroll
	for (int q = 0; q < KPB; ++q) {
		const long k = (k0 + q) % nn;	// frequencies past the list's half length are zeroed below
		ar[q] = 0.0; ai[q] = 0.0;
		idx[q] = (k * tid) % nn;
		stp[q] = (k * HT) % nn;
	}
	for (long j = tid; j < nn; j += HT) {
		const double xv = xi[j];
#pragma unroll
		for (int q = 0; q < KPB; ++q) {
			const double2 tw = wi[idx[q]];
			ar[q] = fma(xv, tw.x, ar[q]);
			ai[q] = fma(xv, tw.y, ai[q]);
			idx[q] += stp[q];
			if (idx[q] >= nn) idx[q] -= nn;
		}
	}
#pragma unroll
	for (int q = 0; q < KPB; ++q) { red[0][q][tid] = ar[q]; red[1][q][tid] = ai[q]; }
	__syncthreads();
	for (int s = HT / 2; s > 0; s >>= 1) {
		if (tid < s)
#pragma unroll
			for (int q = 0; q < KPB; ++q) { red[0][q][tid] += red[0][q][tid + s]; red[1][q][tid] += red[1][q][tid + s]; }
		__syncthreads();
	}
	if (tid < KPB) {
		const long k = k0 + tid;
		if (k >= kmax) return;
		const long nh = (nn + 1) / 2;
		double out = 0.0;
		if (k < nh) {
			const double PI = 3.141592653589793, c = 137.036;
			const double f = dt / (2.0 * PI);
			const double dr = red[0][tid][0] * f, di = red[1][tid][0] * f;
			const double a = dr * dr + di * di;
			const double om = 2.0 * PI / (dt * (double)nn) * (double)k;
			out = (type == 1 ? 4.0 * PI * PI * om * om : (om > 0 ? 4.0 * PI * PI / (om * om) : 0.0)) / (c * c) * a;
		}
		spec[(long)inst * kmax + k] = out;
	}
}

} // namespace
} // namespace qpc

using namespace qpc;

extern "C" int qpc_hhg_spectra(int32_t n_inst, const double* z, int64_t ldz, const int64_t* n, double t0, double dt, const double* tmin,
	const double* tmax, int32_t dipole_type, int64_t kmax, double* spectrum)
{
	if (n_inst < 1 || !z || !n || !tmin || !tmax || !spectrum || kmax < 1 || !(dt > 0) || (dipole_type != 1 && dipole_type != 2)) {
		set_error("qpc_hhg_spectra: bad arguments");
		return QPC_ERR_ARGS;
	}
	long nmax = 0;
	for (int i = 0; i < n_inst; ++i) {
		if (n[i] < 1 || n[i] > ldz || !(tmax[i] > tmin[i])) {
			set_error("qpc_hhg_spectra: list %d: n=%lld ldz=%lld", i, (long long)n[i], (long long)ldz);
			return QPC_ERR_ARGS;
		}
		nmax = std::max<long>(nmax, n[i]);
	}
	if (n_inst > 65535 || (kmax + KPB - 1) / KPB > 2147483647L) { set_error("qpc_hhg_spectra: too many lists or frequencies"); return QPC_ERR_ARGS; }
	int dev = 0;
	if (int rc = check_device(&dev)) return rc;
	// the windowed signal on the host, as qpc_hhg_spectrum forms it
	std::vector<double> x((size_t)n_inst * nmax, 0.0);
	std::vector<long long> nl(n, n + n_inst);
	for (int i = 0; i < n_inst; ++i)
		for (long j = 0; j < n[i]; ++j) {
			const double t = t0 + dt * (double)j;
			const double win = (t > tmin[i] && t < tmax[i]) ? std::pow(std::sin(M_PI * (t - tmin[i]) / (tmax[i] - tmin[i])), 2) : 0.0;
			x[(size_t)i * nmax + j] = -z[(size_t)i * ldz + j] * win;
		}
	cudaStream_t st = nullptr;
	QPC_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
	struct sguard { cudaStream_t s; ~sguard() { cudaStreamDestroy(s); } } sg{st};
	double *dx = nullptr, *ds = nullptr;
	double2* dw = nullptr;
	long long* dn = nullptr;
	// stream-ordered scratch: freed in stream order, so a wait that runs out never blocks on it
	if (cudaMallocAsync((void**)&dx, sizeof(double) * x.size(), st) != cudaSuccess ||
		cudaMallocAsync((void**)&dw, sizeof(double2) * x.size(), st) != cudaSuccess ||
		cudaMallocAsync((void**)&ds, sizeof(double) * (size_t)n_inst * kmax, st) != cudaSuccess ||
		cudaMallocAsync((void**)&dn, sizeof(long long) * n_inst, st) != cudaSuccess) {
		set_error("qpc_hhg_spectra: cudaMallocAsync failed");
		if (dx) cudaFreeAsync(dx, st);
		if (dw) cudaFreeAsync(dw, st);
		if (ds) cudaFreeAsync(ds, st);
		if (dn) cudaFreeAsync(dn, st);
		return QPC_ERR_NOMEM;
	}
	int rc = QPC_OK;
	if (cudaMemcpyAsync(dx, x.data(), sizeof(double) * x.size(), cudaMemcpyHostToDevice, st) != cudaSuccess ||
		cudaMemcpyAsync(dn, nl.data(), sizeof(long long) * n_inst, cudaMemcpyHostToDevice, st) != cudaSuccess) {
		set_error("qpc_hhg_spectra: upload failed");
		rc = QPC_ERR_CUDA;
	}
	if (!rc) {
		k_hhg_twiddle<<<dim3((unsigned)((nmax + 255) / 256), (unsigned)n_inst), 256, 0, st>>>(dn, nmax, dw);
		k_hhg_dft<<<dim3((unsigned)((kmax + KPB - 1) / KPB), (unsigned)n_inst), HT, 0, st>>>(dx, nmax, dw, nmax, dn, kmax, dt, dipole_type, ds);
		if (cudaGetLastError() != cudaSuccess) { set_error("qpc_hhg_spectra: launch failed"); rc = QPC_ERR_CUDA; }
	}
	if (!rc) rc = copy_to_host(spectrum, ds, sizeof(double) * (size_t)n_inst * kmax, st);
	cudaFreeAsync(dx, st);
	cudaFreeAsync(dw, st);
	cudaFreeAsync(ds, st);
	cudaFreeAsync(dn, st);
	if (rc == QPC_OK) rc = wait_on(st);
	return rc;
}
