// Ensemble MLP for the spectra surrogate: members x (n_in -> n_layers x n_hidden GELU
// -> n_out), trained with Adam on the GPU.  No counterpart in the reference.
//
// Numerics: weights and activations enter every product as bfloat16, products are
// accumulated in fp32 on the tensor cores (mma.sync m16n8k16 bf16 -> f32), biases,
// pre-activations, GELU, the loss gradient and the Adam state are fp32, and the
// master weights are fp32 (re-rounded to bf16 after each update).
//
// Every GEMM is C[M][N] = sum_k A[m][k] B[n][k] with both operands k-contiguous:
//   forward   Z = A W^T          A = activations [M][K],  B = W   [N][K]
//   input grad  dA = G W         A = G [M][N],            B = W^T [K][N]
//   weight grad dW = G^T A       A = G^T [N][M],          B = A^T [K][M]
// so each layer keeps its activations and gradients in both orientations, written
// by the epilogue of the kernel that produces them.  One launch covers all members
// (blockIdx.z).
#include "qpc_internal.h"
#include "qpc_cuda_util.cuh"
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cmath>
#include <cstdint>
#include <vector>
#include <algorithm>

namespace qpc {
namespace {

constexpr int MT = 64;          // block tile (rows and columns)
constexpr int MLP_THREADS = 128; // 4 warps, 2 x 2 warp tiles of 32 x 32

enum { EPI_STORE = 0, EPI_HIDDEN = 1, EPI_BACK = 2 };

struct gemm_args {
	const __nv_bfloat16* A; long sA;  // [M][K] per member, member stride
	const __nv_bfloat16* B; long sB;  // [N][K]
	int M, N, K;
	const float* bias; long sbias;    // [N] or null
	const float* aux; long saux;      // EPI_BACK: pre-activation Z [M][N]
	float* out; long sout;            // fp32 [M][N]
	__nv_bfloat16* outb; long soutb;  // bf16 [M][N] (EPI_HIDDEN/EPI_BACK)
	__nv_bfloat16* outt; long soutt;  // bf16 [N][M]
};

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z)
{
	return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16* base, int row, int col, int nrow, int ld)
{
	if (row >= nrow) return 0u;
	return *reinterpret_cast<const uint32_t*>(base + (long)row * ld + col);
}

template <int EPI>
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_gemm(gemm_args a)
{
	const int e = blockIdx.z;
	const __nv_bfloat16* A = a.A + e * a.sA;
	const __nv_bfloat16* B = a.B + e * a.sB;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int gid = lane >> 2, tig = lane & 3;
	const int m0 = blockIdx.y * MT + (warp >> 1) * 32;
	const int n0 = blockIdx.x * MT + (warp & 1) * 32;
	float acc[2][4][4];
#pragma unroll
	for (int i = 0; i < 2; ++i)
#pragma unroll
		for (int j = 0; j < 4; ++j)
#pragma unroll
			for (int c = 0; c < 4; ++c) acc[i][j][c] = 0.f;
	for (int k0 = 0; k0 < a.K; k0 += 16) {
		uint32_t af[2][4], bf[4][2];
#pragma unroll
		for (int i = 0; i < 2; ++i) {
			int r = m0 + i * 16 + gid;
			af[i][0] = ld_pair(A, r, k0 + tig * 2, a.M, a.K);
			af[i][1] = ld_pair(A, r + 8, k0 + tig * 2, a.M, a.K);
			af[i][2] = ld_pair(A, r, k0 + tig * 2 + 8, a.M, a.K);
			af[i][3] = ld_pair(A, r + 8, k0 + tig * 2 + 8, a.M, a.K);
		}
#pragma unroll
		for (int j = 0; j < 4; ++j) {
			int c = n0 + j * 8 + gid;
			bf[j][0] = ld_pair(B, c, k0 + tig * 2, a.N, a.K);
			bf[j][1] = ld_pair(B, c, k0 + tig * 2 + 8, a.N, a.K);
		}
#pragma unroll
		for (int i = 0; i < 2; ++i)
#pragma unroll
			for (int j = 0; j < 4; ++j)
				asm volatile(
					"mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
					: "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
					: "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bf[j][0]), "r"(bf[j][1]));
	}
	// epilogue: acc[i][j][c] is C(row, col) with row = m0+16i+gid+8(c>>1), col = n0+8j+2tig+(c&1)
#pragma unroll
	for (int i = 0; i < 2; ++i)
#pragma unroll
		for (int j = 0; j < 4; ++j)
#pragma unroll
			for (int c = 0; c < 4; ++c) {
				int row = m0 + i * 16 + gid + 8 * (c >> 1);
				int col = n0 + j * 8 + tig * 2 + (c & 1);
				if (row >= a.M || col >= a.N) continue;
				float v = acc[i][j][c];
				long o = (long)row * a.N + col;
				if (a.bias) v += a.bias[e * a.sbias + col];
				if (EPI == EPI_STORE) {
					a.out[e * a.sout + o] = v;
				} else if (EPI == EPI_HIDDEN) {
					a.out[e * a.sout + o] = v;
					__nv_bfloat16 h = __float2bfloat16_rn(gelu(v));
					a.outb[e * a.soutb + o] = h;
					a.outt[e * a.soutt + (long)col * a.M + row] = h;
				} else {
					float d = v * gelu_grad(a.aux[e * a.saux + o]);
					a.out[e * a.sout + o] = d;
					__nv_bfloat16 hb = __float2bfloat16_rn(d);
					a.outb[e * a.soutb + o] = hb;
					a.outt[e * a.soutt + (long)col * a.M + row] = hb;
				}
			}
}

// rows of the dataset into the first layer's input (bf16, zero-padded to K0, both
// orientations) and the targets; idx < 0 marks a padding row (zero input, no loss)
__global__ void k_mlp_gather(const float* __restrict__ X, const float* __restrict__ Y, const int* __restrict__ idx,
	int n_in, int K0, int n_out, int M, __nv_bfloat16* A0, __nv_bfloat16* A0t, float* Yb)
{
	const int e = blockIdx.y;
	const int m = blockIdx.x;
	const int id = idx[e * M + m];
	for (int k = threadIdx.x; k < K0; k += blockDim.x) {
		float v = (id >= 0 && k < n_in) ? X[(long)id * n_in + k] : 0.f;
		__nv_bfloat16 b = __float2bfloat16_rn(v);
		A0[((long)e * M + m) * K0 + k] = b;
		A0t[((long)e * K0 + k) * M + m] = b;
	}
	if (Y)
		for (int k = threadIdx.x; k < n_out; k += blockDim.x) Yb[((long)e * M + m) * n_out + k] = id >= 0 ? Y[(long)id * n_out + k] : 0.f;
}

// G = 2 (Yhat - Y) / (M_valid n_out) on valid rows, 0 on padding rows; per-member sum of
// squared errors, per block then in fixed order by k_mlp_loss_sum
__global__ void k_mlp_loss(const float* __restrict__ Yh, const float* __restrict__ Y, const int* __restrict__ idx, int M, int n_out,
	float scale, long sg, float* G, __nv_bfloat16* Gb, __nv_bfloat16* Gt, float* part)
{
	const int e = blockIdx.y, m = blockIdx.x;
	const bool valid = idx[e * M + m] >= 0;
	__shared__ float sm[32];
	float s = 0.f;
	for (int k = threadIdx.x; k < n_out; k += blockDim.x) {
		long o = ((long)e * M + m) * n_out + k;
		float d = valid ? Yh[o] - Y[o] : 0.f;
		s += d * d;
		float g = 2.f * d * scale;
		long og = e * sg + (long)m * n_out + k;
		G[og] = g;
		__nv_bfloat16 b = __float2bfloat16_rn(g);
		Gb[og] = b;
		Gt[e * sg + (long)k * M + m] = b;
	}
	for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
	if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
	__syncthreads();
	if (threadIdx.x == 0) {
		float t = 0.f;
		for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
		part[e * M + m] = t;
	}
}

__global__ void k_mlp_loss_sum(const float* __restrict__ part, int M, float scale, float* loss)
{
	const int e = blockIdx.x;
	if (threadIdx.x) return;
	double t = 0.0;
	for (int m = 0; m < M; ++m) t += part[e * M + m];
	loss[e] = (float)(t * scale);
}

// gb[n] = sum_m G[m][n], rows in order
__global__ void k_mlp_bias_grad(const float* __restrict__ G, long sg, int M, int N, float* gb, long sgb)
{
	const int e = blockIdx.y;
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if (n >= N) return;
	float s = 0.f;
	for (int m = 0; m < M; ++m) s += G[e * sg + (long)m * N + n];
	gb[e * sgb + n] = s;
}

// Adam (Kingma & Ba 2015) on the fp32 masters of one member's parameters, then the
// bf16 copies of the weights in both orientations
struct adam_layer {
	float *W, *b, *gW, *gb, *mW, *vW, *mb, *vb;
	__nv_bfloat16 *Wb, *Wt;
	int N, K;
};

__global__ void k_mlp_adam(adam_layer L, long sW, long sb, long sWb, float lr, float b1, float b2, float c1, float c2, float eps)
{
	const int e = blockIdx.y;
	const long nw = (long)L.N * L.K;
	for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nw + L.N; i += (long)gridDim.x * blockDim.x) {
		const bool isw = i < nw;
		float* p = isw ? L.W + e * sW + i : L.b + e * sb + (i - nw);
		const float g = isw ? L.gW[e * sW + i] : L.gb[e * sb + (i - nw)];
		float* m = isw ? L.mW + e * sW + i : L.mb + e * sb + (i - nw);
		float* v = isw ? L.vW + e * sW + i : L.vb + e * sb + (i - nw);
		float mm = b1 * *m + (1.f - b1) * g;
		float vv = b2 * *v + (1.f - b2) * g * g;
		*m = mm;
		*v = vv;
		float w = *p - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
		*p = w;
		if (isw) {
			int n = (int)(i / L.K), k = (int)(i - (long)n * L.K);
			__nv_bfloat16 b = __float2bfloat16_rn(w);
			L.Wb[e * sWb + i] = b;
			L.Wt[e * sWb + (long)k * L.N + n] = b;
		}
	}
}

__global__ void k_mlp_cast(const float* __restrict__ W, int N, int K, long sW, __nv_bfloat16* Wb, __nv_bfloat16* Wt)
{
	const int e = blockIdx.y;
	const long nw = (long)N * K;
	for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += (long)gridDim.x * blockDim.x) {
		int n = (int)(i / K), k = (int)(i - (long)n * K);
		__nv_bfloat16 b = __float2bfloat16_rn(W[e * sW + i]);
		Wb[e * sW + i] = b;
		Wt[e * sW + (long)k * N + n] = b;
	}
}

} // namespace
} // namespace qpc

using namespace qpc;

struct qpc_mlp {
	int dev = 0;
	int n_in = 0, K0 = 0, n_hidden = 0, n_layers = 0, n_out = 0, E = 0, J = 0;
	std::vector<int> Ns, Ks;          // per linear layer j: out, in
	std::vector<long> offW, offb;     // offsets of layer j in the per-member flat arrays
	long nW = 0, nb = 0;              // per-member totals
	cudaStream_t st = nullptr;
	float *W = nullptr, *b = nullptr, *gW = nullptr, *gb = nullptr, *mW = nullptr, *vW = nullptr, *mb = nullptr, *vb = nullptr;
	__nv_bfloat16 *Wb = nullptr, *Wt = nullptr;
	long t = 0;                       // Adam step count
	// batch work space (capacity M)
	int Mcap = 0;
	std::vector<__nv_bfloat16*> Act, ActT;  // layer inputs j = 0..J-1: [E][M][K_j] and [E][K_j][M]
	std::vector<float*> Z;                  // pre-activations of hidden layers [E][M][N_j]
	float *Yh = nullptr, *Yb = nullptr, *G = nullptr, *part = nullptr, *loss = nullptr;
	__nv_bfloat16 *Gb = nullptr, *Gt = nullptr;
	int* idx = nullptr;
	// dataset on the device
	float *dX = nullptr, *dY = nullptr;
	long dcap = 0;
};

namespace {

void mlp_free_batch(qpc_mlp* h)
{
	for (auto p : h->Act) cudaFree(p);
	for (auto p : h->ActT) cudaFree(p);
	for (auto p : h->Z) cudaFree(p);
	h->Act.clear(); h->ActT.clear(); h->Z.clear();
	void* ps[] = {h->Yh, h->Yb, h->G, h->part, h->loss, h->Gb, h->Gt, h->idx};
	for (void* p : ps) if (p) cudaFree(p);
	h->Yh = h->Yb = h->G = h->part = h->loss = nullptr;
	h->Gb = h->Gt = nullptr;
	h->idx = nullptr;
	h->Mcap = 0;
}

void mlp_free(qpc_mlp* h)
{
	if (!h) return;
	cudaSetDevice(h->dev);
	mlp_free_batch(h);
	void* ps[] = {h->W, h->b, h->gW, h->gb, h->mW, h->vW, h->mb, h->vb, h->Wb, h->Wt, h->dX, h->dY};
	for (void* p : ps) if (p) cudaFree(p);
	if (h->st) cudaStreamDestroy(h->st);
	delete h;
}

// every kernel of a pass works on exactly Mcap rows (padding rows carry idx < 0)
int ensure_batch(qpc_mlp* h, int M)
{
	if (M == h->Mcap) return QPC_OK;
	mlp_free_batch(h);
	const int E = h->E, J = h->J;
	int rc = 0;
	h->Act.assign(J, nullptr); h->ActT.assign(J, nullptr); h->Z.assign(J, nullptr);
	for (int j = 0; j < J; ++j) {
		if ((rc = dalloc(&h->Act[j], (size_t)E * M * h->Ks[j])) || (rc = dalloc(&h->ActT[j], (size_t)E * M * h->Ks[j]))) return rc;
		if (j < J - 1 && (rc = dalloc(&h->Z[j], (size_t)E * M * h->Ns[j]))) return rc;
	}
	const int maxN = *std::max_element(h->Ns.begin(), h->Ns.end());
	if ((rc = dalloc(&h->Yh, (size_t)E * M * h->n_out)) || (rc = dalloc(&h->Yb, (size_t)E * M * h->n_out)) ||
		(rc = dalloc(&h->G, (size_t)E * M * maxN)) || (rc = dalloc(&h->Gb, (size_t)E * M * maxN)) ||
		(rc = dalloc(&h->Gt, (size_t)E * M * maxN)) || (rc = dalloc(&h->part, (size_t)E * M)) || (rc = dalloc(&h->loss, (size_t)E)) ||
		(rc = dalloc(&h->idx, (size_t)E * M)))
		return rc;
	h->Mcap = M;
	return QPC_OK;
}

// second buffer for the gradient chain: G (fp32/bf16) alternate with the Act-sized
// scratch of the layer below; the backward pass writes layer j-1's gradient into
// dedicated buffers allocated on first use
struct back_bufs {
	float* G2 = nullptr;
	__nv_bfloat16 *G2b = nullptr, *G2t = nullptr;
};

template <int EPI>
void gemm(cudaStream_t st, int E, const __nv_bfloat16* A, long sA, const __nv_bfloat16* B, long sB, int M, int N, int K,
	const float* bias, long sbias, const float* aux, long saux, float* out, long sout, __nv_bfloat16* outb, long soutb,
	__nv_bfloat16* outt, long soutt)
{
	gemm_args a{A, sA, B, sB, M, N, K, bias, sbias, aux, saux, out, sout, outb, soutb, outt, soutt};
	dim3 grid((N + MT - 1) / MT, (M + MT - 1) / MT, E);
	k_mlp_gemm<EPI><<<grid, MLP_THREADS, 0, st>>>(a);
}

// forward of the Mcap rows gathered into Act[0]; output in Yh
void forward(qpc_mlp* h)
{
	const int E = h->E, J = h->J, M = h->Mcap;
	for (int j = 0; j < J; ++j) {
		const int N = h->Ns[j], K = h->Ks[j];
		const __nv_bfloat16* W = h->Wb + h->offW[j];
		if (j < J - 1)
			gemm<EPI_HIDDEN>(h->st, E, h->Act[j], (long)h->Mcap * K, W, h->nW, M, N, K, h->b + h->offb[j], h->nb, nullptr, 0,
				h->Z[j], (long)h->Mcap * N, h->Act[j + 1], (long)h->Mcap * N, h->ActT[j + 1], (long)h->Mcap * N);
		else
			gemm<EPI_STORE>(h->st, E, h->Act[j], (long)h->Mcap * K, W, h->nW, M, N, K, h->b + h->offb[j], h->nb, nullptr, 0,
				h->Yh, (long)h->Mcap * N, nullptr, 0, nullptr, 0);
	}
}

// loss and gradients of the batch in Act[0] / Yb (idx marks valid rows); gW, gb filled
int backward(qpc_mlp* h, int Mvalid, back_bufs& bb)
{
	const int E = h->E, J = h->J, M = h->Mcap;
	const int maxN = *std::max_element(h->Ns.begin(), h->Ns.end());
	if (!bb.G2) {
		// stream-ordered: freed in stream order by free_back, which never blocks
		const size_t n = (size_t)E * h->Mcap * maxN;
		if (cudaMallocAsync((void**)&bb.G2, sizeof(float) * n, h->st) != cudaSuccess ||
			cudaMallocAsync((void**)&bb.G2b, sizeof(__nv_bfloat16) * n, h->st) != cudaSuccess ||
			cudaMallocAsync((void**)&bb.G2t, sizeof(__nv_bfloat16) * n, h->st) != cudaSuccess) {
			set_error("cudaMallocAsync of the gradient scratch failed");
			return QPC_ERR_NOMEM;
		}
	}
	const float scale = 1.0f / ((float)Mvalid * (float)h->n_out);
	const long sg = (long)h->Mcap * maxN;
	k_mlp_loss<<<dim3(M, E), 128, 0, h->st>>>(h->Yh, h->Yb, h->idx, M, h->n_out, scale, sg, h->G, h->Gb, h->Gt, h->part);
	k_mlp_loss_sum<<<E, 32, 0, h->st>>>(h->part, h->Mcap, scale, h->loss);
	float* G = h->G;
	__nv_bfloat16 *Gb = h->Gb, *Gt = h->Gt;
	float* G2 = bb.G2;
	__nv_bfloat16 *G2b = bb.G2b, *G2t = bb.G2t;
	for (int j = J - 1; j >= 0; --j) {
		const int N = h->Ns[j], K = h->Ks[j];
		// gW_j[n][k] = sum_m G[m][n] A_j[m][k]: A = G^T [N][M], B = A_j^T [K][M]
		gemm<EPI_STORE>(h->st, E, Gt, sg, h->ActT[j], (long)h->Mcap * K, N, K, M, nullptr, 0, nullptr, 0,
			h->gW + h->offW[j], h->nW, nullptr, 0, nullptr, 0);
		k_mlp_bias_grad<<<dim3((N + 127) / 128, E), 128, 0, h->st>>>(G, sg, M, N, h->gb + h->offb[j], h->nb);
		if (j > 0) {
			// dA[m][k] = sum_n G[m][n] W[n][k]: A = G [M][N], B = W^T [K][N]; times gelu'(Z_{j-1})
			gemm<EPI_BACK>(h->st, E, Gb, sg, h->Wt + h->offW[j], h->nW, M, K, N, nullptr, 0, h->Z[j - 1], (long)h->Mcap * K,
				G2, sg, G2b, sg, G2t, sg);
			std::swap(G, G2); std::swap(Gb, G2b); std::swap(Gt, G2t);
		}
	}
	return QPC_OK;
}

void adam(qpc_mlp* h, float lr)
{
	const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
	h->t += 1;
	const float c1 = 1.f - powf(b1, (float)h->t), c2 = 1.f - powf(b2, (float)h->t);
	for (int j = 0; j < h->J; ++j) {
		adam_layer L{h->W + h->offW[j], h->b + h->offb[j], h->gW + h->offW[j], h->gb + h->offb[j], h->mW + h->offW[j], h->vW + h->offW[j],
			h->mb + h->offb[j], h->vb + h->offb[j], h->Wb + h->offW[j], h->Wt + h->offW[j], h->Ns[j], h->Ks[j]};
		long n = (long)h->Ns[j] * h->Ks[j] + h->Ns[j];
		int blocks = (int)std::min<long>((n + 255) / 256, 1024);
		k_mlp_adam<<<dim3(blocks, h->E), 256, 0, h->st>>>(L, h->nW, h->nb, h->nW, lr, b1, b2, c1, c2, eps);
	}
}

void cast_all(qpc_mlp* h)
{
	for (int j = 0; j < h->J; ++j) {
		long nw = (long)h->Ns[j] * h->Ks[j];
		k_mlp_cast<<<dim3((int)std::min<long>((nw + 255) / 256, 1024), h->E), 256, 0, h->st>>>(h->W + h->offW[j], h->Ns[j], h->Ks[j],
			h->nW, h->Wb + h->offW[j], h->Wt + h->offW[j]);
	}
}

// splitmix64 (Steele, Lea and Flood 2014) for the initial weights
uint64_t splitmix(uint64_t& s)
{
	uint64_t z = (s += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

int upload_data(qpc_mlp* h, const float* X, const float* Y, long n)
{
	if (n > h->dcap) {
		if (h->dX) cudaFree(h->dX);
		if (h->dY) cudaFree(h->dY);
		h->dX = h->dY = nullptr; h->dcap = 0;
		int rc;
		if ((rc = dalloc(&h->dX, (size_t)n * h->n_in)) || (rc = dalloc(&h->dY, (size_t)n * h->n_out))) return rc;
		h->dcap = n;
	}
	QPC_CUDA(cudaMemcpyAsync(h->dX, X, sizeof(float) * n * h->n_in, cudaMemcpyHostToDevice, h->st));
	if (Y) QPC_CUDA(cudaMemcpyAsync(h->dY, Y, sizeof(float) * n * h->n_out, cudaMemcpyHostToDevice, h->st));
	return QPC_OK;
}

void free_back(back_bufs& bb, cudaStream_t st)
{
	if (bb.G2) cudaFreeAsync(bb.G2, st);
	if (bb.G2b) cudaFreeAsync(bb.G2b, st);
	if (bb.G2t) cudaFreeAsync(bb.G2t, st);
	bb = back_bufs{};
}

int round_m(int m) { return (m + MT - 1) / MT * MT; }

} // namespace

extern "C" {

int qpc_mlp_create(int32_t n_in, int32_t n_hidden, int32_t n_layers, int32_t n_out, int32_t n_members, uint64_t seed, qpc_mlp** out)
{
	if (!out) { set_error("out is NULL"); return QPC_ERR_ARGS; }
	*out = nullptr;
	if (n_in < 1 || n_hidden < 16 || n_hidden % 16 || n_layers < 1 || n_out < 8 || n_out % 8 || n_members < 1 || n_members > 64) {
		set_error("bad MLP shape n_in=%d n_hidden=%d n_layers=%d n_out=%d members=%d (hidden a multiple of 16, out of 8)",
			n_in, n_hidden, n_layers, n_out, n_members);
		return QPC_ERR_ARGS;
	}
	int dev = 0;
	if (int rc = check_device(&dev)) return rc;
	qpc_mlp* h = new (std::nothrow) qpc_mlp;
	if (!h) { set_error("host allocation"); return QPC_ERR_NOMEM; }
	auto fail = [&](int rc) { mlp_free(h); return rc; };
	h->dev = dev;
	h->n_in = n_in; h->K0 = (n_in + 15) / 16 * 16; h->n_hidden = n_hidden; h->n_layers = n_layers; h->n_out = n_out;
	h->E = n_members; h->J = n_layers + 1;
	for (int j = 0; j < h->J; ++j) {
		h->Ks.push_back(j == 0 ? h->K0 : n_hidden);
		h->Ns.push_back(j == h->J - 1 ? n_out : n_hidden);
		h->offW.push_back(h->nW);
		h->offb.push_back(h->nb);
		h->nW += (long)h->Ns[j] * h->Ks[j];
		h->nb += h->Ns[j];
	}
	if ((cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking)) != cudaSuccess) { set_error("cudaStreamCreateWithFlags failed"); return fail(QPC_ERR_CUDA); }
	const size_t tw = (size_t)h->E * h->nW, tb = (size_t)h->E * h->nb;
	int rc;
	if ((rc = dalloc(&h->W, tw)) || (rc = dalloc(&h->b, tb)) || (rc = dalloc(&h->gW, tw)) || (rc = dalloc(&h->gb, tb)) ||
		(rc = dalloc(&h->mW, tw)) || (rc = dalloc(&h->vW, tw)) || (rc = dalloc(&h->mb, tb)) || (rc = dalloc(&h->vb, tb)) ||
		(rc = dalloc(&h->Wb, tw)) || (rc = dalloc(&h->Wt, tw)))
		return fail(rc);
	// He-uniform weights (bound sqrt(6 / fan_in), fan_in = the unpadded inputs), zero biases
	std::vector<float> W(tw, 0.f);
	uint64_t sd = seed;
	for (int e = 0; e < h->E; ++e)
		for (int j = 0; j < h->J; ++j) {
			const int fan = j == 0 ? n_in : h->Ks[j];
			const float bound = std::sqrt(6.0f / (float)fan);
			for (int nn = 0; nn < h->Ns[j]; ++nn)
				for (int k = 0; k < h->Ks[j]; ++k) {
					double u = (double)(splitmix(sd) >> 11) * (1.0 / 9007199254740992.0);
					W[(size_t)e * h->nW + h->offW[j] + (size_t)nn * h->Ks[j] + k] = (j == 0 && k >= n_in) ? 0.f : (float)((2.0 * u - 1.0) * bound);
				}
		}
	if (cudaMemcpy(h->W, W.data(), sizeof(float) * tw, cudaMemcpyHostToDevice) != cudaSuccess ||
		cudaMemset(h->b, 0, sizeof(float) * tb) != cudaSuccess || cudaMemset(h->mW, 0, sizeof(float) * tw) != cudaSuccess ||
		cudaMemset(h->vW, 0, sizeof(float) * tw) != cudaSuccess || cudaMemset(h->mb, 0, sizeof(float) * tb) != cudaSuccess ||
		cudaMemset(h->vb, 0, sizeof(float) * tb) != cudaSuccess) {
		set_error("device upload failed");
		return fail(QPC_ERR_CUDA);
	}
	cast_all(h);
	if (cudaGetLastError() != cudaSuccess) { set_error("cast failed"); return fail(QPC_ERR_CUDA); }
	if (int rc2 = wait_on(h->st)) return fail(rc2);
	*out = h;
	return QPC_OK;
}

int qpc_mlp_destroy(qpc_mlp* h)
{
	mlp_free(h);
	return QPC_OK;
}

int qpc_mlp_param_count(qpc_mlp* h, int64_t* n)
{
	if (!h || !n) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	*n = h->nW + h->nb;
	return QPC_OK;
}

// flat fp32 parameters of one member: W_0 [N][K0] (K0 = n_in rounded up to 16, padding
// columns ignored on set and zero on get), b_0, W_1, b_1, ...
static int params_io(qpc_mlp* h, int32_t member, float* host, bool get)
{
	if (!h || !host || member < 0 || member >= h->E) { set_error("bad arguments"); return QPC_ERR_ARGS; }
	cudaSetDevice(h->dev);
	long o = 0;
	for (int j = 0; j < h->J; ++j) {
		const size_t nw = (size_t)h->Ns[j] * h->Ks[j];
		float* dW = h->W + (size_t)member * h->nW + h->offW[j];
		float* db = h->b + (size_t)member * h->nb + h->offb[j];
		if (get) {
			QPC_CUDA(cudaMemcpy(host + o, dW, sizeof(float) * nw, cudaMemcpyDeviceToHost));
			QPC_CUDA(cudaMemcpy(host + o + nw, db, sizeof(float) * h->Ns[j], cudaMemcpyDeviceToHost));
		} else {
			std::vector<float> w(host + o, host + o + nw);
			if (j == 0)
				for (int nn = 0; nn < h->Ns[j]; ++nn)
					for (int k = h->n_in; k < h->K0; ++k) w[(size_t)nn * h->K0 + k] = 0.f;
			QPC_CUDA(cudaMemcpy(dW, w.data(), sizeof(float) * nw, cudaMemcpyHostToDevice));
			QPC_CUDA(cudaMemcpy(db, host + o + nw, sizeof(float) * h->Ns[j], cudaMemcpyHostToDevice));
		}
		o += nw + h->Ns[j];
	}
	if (!get) {
		cast_all(h);
		QPC_CUDA(cudaGetLastError());
		if (int rc = wait_on(h->st)) return rc;
	}
	return QPC_OK;
}

int qpc_mlp_get_params(qpc_mlp* h, int32_t member, float* params) { return params_io(h, member, params, true); }
int qpc_mlp_set_params(qpc_mlp* h, int32_t member, const float* params) { return params_io(h, member, const_cast<float*>(params), false); }

// loss and gradient of every member on the same n rows (no update); grad [members][param_count]
int qpc_mlp_loss_grad(qpc_mlp* h, const float* X, const float* Y, int32_t n, float* loss, float* grad)
{
	if (!h || !X || !Y || !loss || n < 1) { set_error("bad arguments"); return QPC_ERR_ARGS; }
	cudaSetDevice(h->dev);
	const int M = round_m(n);
	if (int rc = ensure_batch(h, M)) return rc;
	if (int rc = upload_data(h, X, Y, n)) return rc;
	std::vector<int> idx((size_t)h->E * h->Mcap, -1);
	for (int e = 0; e < h->E; ++e)
		for (int m = 0; m < n; ++m) idx[(size_t)e * h->Mcap + m] = m;
	QPC_CUDA(cudaMemcpyAsync(h->idx, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, h->st));
	k_mlp_gather<<<dim3(M, h->E), 64, 0, h->st>>>(h->dX, h->dY, h->idx, h->n_in, h->K0, h->n_out, M, h->Act[0], h->ActT[0], h->Yb);
	forward(h);
	back_bufs bb;
	int rc = backward(h, n, bb);
	if (!rc && cudaGetLastError() != cudaSuccess) { set_error("kernel launch failed"); rc = QPC_ERR_CUDA; }
	if (!rc) rc = wait_on(h->st);
	if (rc) { free_back(bb, h->st); return rc; }
	free_back(bb, h->st);
	if (int rc2 = copy_to_host(loss, h->loss, sizeof(float) * h->E, h->st)) return rc2;
	if (grad) {
		const long np = h->nW + h->nb;
		std::vector<float> gw((size_t)h->E * h->nW), gbv((size_t)h->E * h->nb);
		if (int rc2 = copy_to_host(gw.data(), h->gW, sizeof(float) * gw.size(), h->st)) return rc2;
		if (int rc2 = copy_to_host(gbv.data(), h->gb, sizeof(float) * gbv.size(), h->st)) return rc2;
		for (int e = 0; e < h->E; ++e) {
			long o = 0;
			for (int j = 0; j < h->J; ++j) {
				const size_t nw = (size_t)h->Ns[j] * h->Ks[j];
				std::copy(gw.begin() + (size_t)e * h->nW + h->offW[j], gw.begin() + (size_t)e * h->nW + h->offW[j] + nw, grad + e * np + o);
				std::copy(gbv.begin() + (size_t)e * h->nb + h->offb[j], gbv.begin() + (size_t)e * h->nb + h->offb[j] + h->Ns[j], grad + e * np + o + nw);
				o += nw + h->Ns[j];
			}
		}
	}
	return QPC_OK;
}

// epochs of Adam over n rows in batches; every member sees its own shuffle (seeded)
// of all rows.  loss_hist [epochs][members] (may be NULL): mean batch loss per epoch.
int qpc_mlp_train(qpc_mlp* h, const float* X, const float* Y, int32_t n, int32_t epochs, int32_t batch, float lr, uint64_t seed,
	float* loss_hist)
{
	if (!h || !X || !Y || n < 1 || epochs < 0 || batch < 1 || !(lr > 0)) { set_error("bad arguments"); return QPC_ERR_ARGS; }
	cudaSetDevice(h->dev);
	const int M = round_m(std::min(batch, n));
	if (int rc = ensure_batch(h, M)) return rc;
	if (int rc = upload_data(h, X, Y, n)) return rc;
	const int nbat = (n + batch - 1) / batch;
	std::vector<int> perm((size_t)h->E * n), idx((size_t)h->E * h->Mcap);
	std::vector<float> lsum(h->E), lb(h->E);
	uint64_t sd = seed;
	back_bufs bb;
	int rc = QPC_OK;
	for (int ep = 0; ep < epochs && !rc; ++ep) {
		for (int e = 0; e < h->E; ++e) {
			int* p = perm.data() + (size_t)e * n;
			for (int i = 0; i < n; ++i) p[i] = i;
			for (int i = n - 1; i > 0; --i) std::swap(p[i], p[splitmix(sd) % (uint64_t)(i + 1)]);
		}
		std::fill(lsum.begin(), lsum.end(), 0.f);
		for (int bi = 0; bi < nbat && !rc; ++bi) {
			const int m0 = bi * batch, mv = std::min(batch, n - m0);
			for (int e = 0; e < h->E; ++e)
				for (int m = 0; m < h->Mcap; ++m) idx[(size_t)e * h->Mcap + m] = m < mv ? perm[(size_t)e * n + m0 + m] : -1;
			if (cudaMemcpyAsync(h->idx, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, h->st) != cudaSuccess) { rc = QPC_ERR_CUDA; break; }
			k_mlp_gather<<<dim3(M, h->E), 64, 0, h->st>>>(h->dX, h->dY, h->idx, h->n_in, h->K0, h->n_out, M, h->Act[0], h->ActT[0], h->Yb);
			forward(h);
			if ((rc = backward(h, mv, bb))) break;
			adam(h, lr);
			if (loss_hist) {
				if ((rc = copy_to_host(lb.data(), h->loss, sizeof(float) * h->E, h->st))) break;
				for (int e = 0; e < h->E; ++e) lsum[e] += lb[e] / nbat;
			}
		}
		if (loss_hist) for (int e = 0; e < h->E; ++e) loss_hist[(size_t)ep * h->E + e] = lsum[e];
	}
	if (!rc && cudaGetLastError() != cudaSuccess) { rc = QPC_ERR_CUDA; set_error("training step failed on the device"); }
	if (!rc) rc = wait_on(h->st);
	free_back(bb, h->st);
	return rc;
}

// every member's prediction for n rows: out [members][n][n_out]
int qpc_mlp_predict(qpc_mlp* h, const float* X, int32_t n, float* out)
{
	if (!h || !X || !out || n < 0) { set_error("bad arguments"); return QPC_ERR_ARGS; }
	if (n == 0) return QPC_OK;
	cudaSetDevice(h->dev);
	const int M = round_m(std::min(1024, n));
	if (int rc = ensure_batch(h, M)) return rc;
	if (int rc = upload_data(h, X, nullptr, n)) return rc;
	std::vector<int> idx((size_t)h->E * h->Mcap);
	std::vector<float> yh((size_t)h->E * h->Mcap * h->n_out);
	for (int m0 = 0; m0 < n; m0 += h->Mcap) {
		const int mv = std::min(h->Mcap, n - m0);
		for (int e = 0; e < h->E; ++e)
			for (int m = 0; m < h->Mcap; ++m) idx[(size_t)e * h->Mcap + m] = m < mv ? m0 + m : -1;
		QPC_CUDA(cudaMemcpyAsync(h->idx, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, h->st));
		k_mlp_gather<<<dim3(M, h->E), 64, 0, h->st>>>(h->dX, nullptr, h->idx, h->n_in, h->K0, h->n_out, M, h->Act[0], h->ActT[0], nullptr);
		forward(h);
		QPC_CUDA(cudaGetLastError());
		if (int rc = copy_to_host(yh.data(), h->Yh, sizeof(float) * yh.size(), h->st)) return rc;
		for (int e = 0; e < h->E; ++e)
			for (int m = 0; m < mv; ++m)
				std::copy(yh.begin() + ((size_t)e * h->Mcap + m) * h->n_out, yh.begin() + ((size_t)e * h->Mcap + m + 1) * h->n_out,
					out + ((size_t)e * n + m0 + m) * h->n_out);
	}
	return QPC_OK;
}

} // extern "C"
