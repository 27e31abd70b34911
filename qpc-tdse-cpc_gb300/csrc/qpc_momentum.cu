// Photoelectron momentum spectra on the GPU: the PCS projector of spectrum_c_pcs
// (measure_lmd / measure_prj / measure_pad, spherical/spectrum/momentum_1e.hpp:337-403)
// and the t-SURFF accumulator of spectrum_c_tsf (accumulate, momentum_1e.hpp:627-777),
// for a batch of wavefunctions c[inst][m][l][r] (complex128).  The tables come from
// qpc_pcs_tables / qpc_tsurff_tables (qpc_momentum.cpp).
//
// Work per call (FP64; channels N_ch = n_m n_l, l = |m| + il):
//   PCS   projections  nkr * n_inst * N_ch * n_r real x complex products (the bulk),
//         then nkr * nkt * nkp * N_ch per instance for PMD (nkr * nkt * N_ch for PAD);
//   tSURF per step: the surface values (N_ch * nb), the flux term per (kr, channel), the
//         l-sum against Y_lm (nkr * nkt * N_ch per instance) and the m-sum with the Volkov
//         phase (nkr * nkt * nkp * n_m per instance).
// Every kernel is a plain FP64 loop: one thread per output element, operands staged in
// shared memory where a block shares them.
#include "qpc_cuda_util.cuh"
#include <cmath>
#include <vector>

using namespace qpc;

namespace {

const double SQRT_2_OVER_PI = 0.797884560802865;	// the literal of momentum_1e.hpp:352 and 664

inline int lmax_of(const qpc_dims& d)
{
	const int m1 = d.m0 + d.n_m - 1;
	return std::max(std::abs(d.m0), std::abs(m1)) + d.n_l - 1;
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }

// ---------------------------------------------------------------- PCS projector
// Q[inst][kr][ch] = cps[kr][l] sum_r ijl[l][r][kr] c[inst][ch][r] for a block of PG instances, one
// channel ch = im n_l + il (l = |m| + il) and 128 consecutive kr; the radial vectors of the
// block's instances are staged in shared memory chunk by chunk.  Grid (instance group, kr tile,
// channel) with the instance group fastest: the blocks that read one slice of ijl run together,
// so the slice is read from HBM once and from L2 by the other instance groups.
constexpr int PG = 8, PCH = 128;
__global__ void __launch_bounds__(128) k_pcs_proj(const double* __restrict__ ijlT, const double2* __restrict__ cps, const double2* __restrict__ c,
	double2* __restrict__ Q, int nkr, int n_r, int n_l, int m0, int nch, int nl_tot, int n_inst)
{
	__shared__ double2 cs[PG][PCH];
	const int kr = blockIdx.y * 128 + threadIdx.x;
	const int ch = blockIdx.z, i0 = blockIdx.x * PG;
	const int im = ch / n_l, il = ch % n_l, l = abs(m0 + im) + il;
	const double* a = ijlT + (size_t)l * n_r * nkr;
	double2 acc[PG];
#pragma unroll
	for (int g = 0; g < PG; ++g) acc[g] = make_double2(0.0, 0.0);
	for (int r0 = 0; r0 < n_r; r0 += PCH) {
		__syncthreads();
		for (int g = 0; g < PG; ++g) {
			const int inst = i0 + g, r = r0 + threadIdx.x;
			cs[g][threadIdx.x] = (inst < n_inst && r < n_r) ? c[((size_t)inst * nch + ch) * n_r + r] : make_double2(0.0, 0.0);
		}
		__syncthreads();
		if (kr < nkr) {
			const int nr = min(PCH, n_r - r0);
			for (int j = 0; j < nr; ++j) {
				const double v = a[(size_t)(r0 + j) * nkr + kr];
#pragma unroll
				for (int g = 0; g < PG; ++g) { acc[g].x += v * cs[g][j].x; acc[g].y += v * cs[g][j].y; }
			}
		}
	}
	if (kr < nkr) {
		const double2 cp = cps[(size_t)kr * nl_tot + l];
		for (int g = 0; g < PG; ++g)
			if (i0 + g < n_inst) Q[((size_t)(i0 + g) * nkr + kr) * nch + ch] = cmul(cp, acc[g]);
	}
}

// With Q = cps <ijl|c> from k_pcs_proj:
// LMD[inst][kr][ch] = sqrt(2/pi) Q                                   (measure_lmd, 386-403)
// PMD[inst][kr][kt][kp] = sqrt(2/pi) sum_m exm[kp][m] sum_l plm Q     (measure_prj, 337-355)
// PAD[inst][kr][kt] = 2 sqrt(kr) sum_m sum_l plm Q                    (measure_pad, 358-383)
// The l-sums are real x complex; the reference's per-term product plm exm cps <ijl|c> is the same
// sum regrouped.
__global__ void k_pcs_out(int kind, const double2* __restrict__ Q, const double* __restrict__ plm, const double2* __restrict__ exm,
	const double* __restrict__ kr, double2* __restrict__ out, int nkr, int nkt, int nkp, int n_l, int n_m, long total)
{
	const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (idx >= total) return;
	const int nch = n_m * n_l;
	if (kind == QPC_SPEC_LMD) {
		out[idx] = cscale(Q[idx], SQRT_2_OVER_PI);
		return;
	}
	const int per_kr = kind == QPC_SPEC_PMD ? nkt * nkp : nkt;
	const int ia = (int)(idx % per_kr);
	const long ikr = (idx / per_kr) % nkr, inst = idx / ((long)per_kr * nkr);
	const int kt = kind == QPC_SPEC_PMD ? ia / nkp : ia, kp = kind == QPC_SPEC_PMD ? ia % nkp : 0;
	const double2* q = Q + (inst * nkr + ikr) * nch;
	const double* pl = plm + (size_t)kt * nch;
	double2 tmp = make_double2(0.0, 0.0);
	for (int im = 0; im < n_m; ++im) {
		double2 v = make_double2(0.0, 0.0);
		for (int il = 0; il < n_l; ++il) {
			const double p = pl[im * n_l + il];
			const double2 x = q[im * n_l + il];
			v.x += p * x.x;
			v.y += p * x.y;
		}
		tmp = kind == QPC_SPEC_PMD ? cadd(tmp, cmul(exm[(size_t)kp * n_m + im], v)) : cadd(tmp, v);
	}
	out[idx] = kind == QPC_SPEC_PMD ? cscale(tmp, SQRT_2_OVER_PI) : cscale(tmp, sqrt(kr[ikr]) * 2.0);
}

// ---------------------------------------------------------------- t-SURFF
// temp[inst][ch] = sum_i c[inst][ch][ib_i] b0_i, temq = the same with br_i (prepare, 606-619)
__global__ void k_ts_prepare(const double2* __restrict__ c, const int* __restrict__ ib, const double* __restrict__ b0,
	const double* __restrict__ br, int nb, int n_r, long total, double2* __restrict__ temp, double2* __restrict__ temq)
{
	const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (idx >= total) return;
	const double2* v = c + idx * n_r;
	double2 s0 = make_double2(0.0, 0.0), s1 = make_double2(0.0, 0.0);
	for (int i = 0; i < nb; ++i) {
		const double2 x = v[ib[i]];
		s0 = cadd(s0, cscale(x, b0[i]));
		s1 = cadd(s1, cscale(x, br[i]));
	}
	temp[idx] = s0;
	temq[idx] = s1;
}

// the same surface values from the length-gauge engine's resident state: r-major [slot][m][r][l],
// instance inst at slot[inst]; temp/temq in the handle's order [inst][m][l]
__global__ void k_ts_prepare_eng(const double2* __restrict__ st, const int* __restrict__ slot, const int* __restrict__ ib,
	const double* __restrict__ b0, const double* __restrict__ br, int nb, int M, int N, int L, long total, double2* __restrict__ temp,
	double2* __restrict__ temq)
{
	const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (idx >= total) return;
	const int l = (int)(idx % L);
	const long im_inst = idx / L;
	const int m = (int)(im_inst % M);
	const long inst = im_inst / M;
	const double2* v = st + ((long)slot[inst] * M + m) * (long)N * L + l;
	double2 s0 = make_double2(0.0, 0.0), s1 = make_double2(0.0, 0.0);
	for (int i = 0; i < nb; ++i) {
		const double2 x = v[(long)ib[i] * L];
		s0 = cadd(s0, cscale(x, b0[i]));
		s1 = cadd(s1, cscale(x, br[i]));
	}
	temp[idx] = s0;
	temq[idx] = s1;
}

// U[inst][kr][ch] = (-i)^(l+1) times the flux term of one channel (accumulate, 627-777):
//   jdb = -1/2 (j0 temq - jr temp);  z adds -i A_z(t_i+1) j0 (temp(l-1) <l-1|cos|l> + temp(l+1) <l|cos|l+1>);
//   xy adds the (m -+ 1, l -+ 1) neighbours with ias = i (A_x - i A_y)/2, iap = i (A_x + i A_y)/2.
__global__ void k_ts_u(int mode, const double2* __restrict__ temp, const double2* __restrict__ temq, const double* __restrict__ j0,
	const double* __restrict__ jr, const double* __restrict__ pm0, const double* __restrict__ pm1, const double* __restrict__ pm2,
	const double* __restrict__ a1, int nkr, int n_l, int n_m, int m0, int nl_tot, long total, double2* __restrict__ U)
{
	const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (idx >= total) return;
	const int nch = n_m * n_l;
	const int ch = (int)(idx % nch);
	const long ikr = (idx / nch) % nkr, inst = idx / ((long)nch * nkr);
	const int im = ch / n_l, il = ch % n_l, am = abs(m0 + im), l = am + il;
	const double2* tp = temp + inst * nch;
	const double J0 = j0[ikr * nl_tot + l], JR = jr[ikr * nl_tot + l];
	const double2 b0v = tp[ch], brv = temq[inst * nch + ch];
	double2 s = cscale(csub(cscale(brv, J0), cscale(b0v, JR)), -0.5);
	if (mode == QPC_TSURFF_Z) {
		const double az = a1[inst];	// A_z(t_i+1)
		const double2 iaz = make_double2(0.0, az);
		const double2 prev = il > 0 ? cscale(cscale(tp[ch - 1], J0), pm0[ch - 1]) : make_double2(0.0, 0.0);
		const double2 next = il + 1 < n_l ? cscale(cscale(tp[ch + 1], J0), pm0[ch]) : make_double2(0.0, 0.0);
		s = csub(csub(s, cmul(iaz, prev)), cmul(iaz, next));
	} else if (mode == QPC_TSURFF_XY) {
		const double ax = a1[2 * inst], ay = a1[2 * inst + 1];	// A_x(t_i+1), A_y(t_i+1)
		const double2 iap = cscale(cmul(make_double2(ax, ay), make_double2(0.0, 1.0)), 0.5);
		const double2 ias = cscale(cmul(make_double2(ax, -ay), make_double2(0.0, 1.0)), 0.5);
		for (int dm = -1; dm <= 1; dm += 2)
			for (int dl = -1; dl <= 1; dl += 2) {
				const int jm = im + dm;
				if (jm < 0 || jm >= n_m) continue;
				const int jl = l + dl - abs(m0 + jm);
				if (jl < 0 || jl >= n_l) continue;
				const int jc = jm * n_l + jl;
				// the four couplings of momentum_1e.hpp:737-752, with the angular element of the lower-m channel
				const double pe = dm < 0 ? (dl < 0 ? pm1[jc] : pm2[jc]) : (dl < 0 ? pm2[ch] : pm1[ch]);
				const double2 w = cscale(cscale(tp[jc], J0), pe);
				s = csub(s, cmul(dm < 0 ? ias : iap, w));
			}
	}
	// (-i)^(l+1)
	const int q = (l + 1) & 3;
	const double2 r = q == 0 ? s : q == 1 ? make_double2(s.y, -s.x) : q == 2 ? make_double2(-s.x, -s.y) : make_double2(-s.y, s.x);
	U[idx] = r;
}

// W[inst][kr][kt][im] = sum_il y0[im][il][kt] U[inst][kr][im][il]; the block's U row in shared memory
__global__ void k_ts_w(const double2* __restrict__ U, const double* __restrict__ y0T, int nkr, int nkt, int n_l, int n_m,
	double2* __restrict__ W)
{
	extern __shared__ double2 us[];
	const int kt = blockIdx.x * blockDim.x + threadIdx.x;
	const int ikr = blockIdx.y, z = blockIdx.z, im = z % n_m, inst = z / n_m;
	const int nch = n_m * n_l;
	const double2* u = U + ((size_t)inst * nkr + ikr) * nch + (size_t)im * n_l;
	for (int il = threadIdx.x; il < n_l; il += blockDim.x) us[il] = u[il];
	__syncthreads();
	if (kt >= nkt) return;
	const double* y = y0T + (size_t)im * n_l * nkt + kt;
	double2 s = make_double2(0.0, 0.0);
	for (int il = 0; il < n_l; ++il) {
		const double v = y[(size_t)il * nkt];
		s.x += v * us[il].x;
		s.y += v * us[il].y;
	}
	W[(((size_t)inst * nkr + ikr) * nkt + kt) * n_m + im] = s;
}

// work[inst][kr][kt][kp] += (sum_im e0[kp][im] W) exp(i phase) dt sqrt(2/pi), with the phase of the
// mode (0.5 k^2 t plus k.(displacement) over the axes the mode carries); clock[inst] = (t, dx, dy, dz)
__global__ void k_ts_acc(int mode, const double2* __restrict__ W, const double2* __restrict__ e0, const double* __restrict__ kr,
	const double* __restrict__ coskt, const double* __restrict__ sinkt, const double* __restrict__ coskp, const double* __restrict__ sinkp,
	const double* __restrict__ clock, double dt, int nkr, int nkt, int nkp, int n_m, long total, double2* __restrict__ work,
	const int* __restrict__ act = nullptr)
{
	const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (idx >= total) return;
	const int kp = (int)(idx % nkp), kt = (int)((idx / nkp) % nkt);
	const long ikr = (idx / ((long)nkp * nkt)) % nkr, inst = idx / ((long)nkp * nkt * nkr);
	if (act && !act[inst]) return;	// this instance takes no accumulate now
	const double2* w = W + ((inst * nkr + ikr) * nkt + kt) * n_m;
	double2 s = make_double2(0.0, 0.0);
	for (int im = 0; im < n_m; ++im) s = cadd(s, cmul(e0[(size_t)kp * n_m + im], w[im]));
	const double k = kr[ikr];
	const double* ck = clock + 4 * inst;
	// rounded as written in the reference, without contraction into FMAs
	double ph = __dmul_rn(__dmul_rn(__dmul_rn(0.5, k), k), ck[0]);
	if (mode != QPC_TSURFF_Z) {
		ph = __dadd_rn(ph, __dmul_rn(__dmul_rn(__dmul_rn(k, sinkt[kt]), coskp[kp]), ck[1]));
		ph = __dadd_rn(ph, __dmul_rn(__dmul_rn(__dmul_rn(k, sinkt[kt]), sinkp[kp]), ck[2]));
	}
	if (mode != QPC_TSURFF_XY) ph = __dadd_rn(ph, __dmul_rn(__dmul_rn(k, coskt[kt]), ck[3]));
	double sn, cs;
	sincos(ph, &sn, &cs);
	const double2 t = cscale(cscale(cmul(s, make_double2(cs, sn)), dt), SQRT_2_OVER_PI);
	work[idx] = cadd(work[idx], t);
}

template <class T> int upload(T** d, const T* h, size_t n)
{
	if (int rc = dalloc(d, n)) return rc;
	QPC_CUDA(cudaMemcpy(*d, h, sizeof(T) * n, cudaMemcpyHostToDevice));
	return QPC_OK;
}

int grid_ok(const qpc_dims* d, const qpc_kgrid* g)
{
	return d && g && d->n_r >= 1 && d->n_l >= 1 && d->n_m >= 1 && g->nkr >= 1 && g->nkt >= 1 && g->nkp >= 1;
}

}  // namespace

struct qpc_pcs {
	int dev = 0;
	qpc_dims d{};
	int nkr = 0, nkt = 0, nkp = 0, nl = 0;
	cudaStream_t st = nullptr;
	cudaEvent_t ev0 = nullptr, ev1 = nullptr;	// bracket the kernels of the last measurement
	float last_ms = 0.f;
	double *ijlT = nullptr, *plm = nullptr, *kr = nullptr;
	double2 *exm = nullptr, *cps = nullptr;
	double2 *cbuf = nullptr, *Q = nullptr, *out = nullptr;
	long cap_c = 0, cap_q = 0, cap_o = 0;
};

struct qpc_tsurff {
	int dev = 0;
	qpc_dims d{};
	int nkr = 0, nkt = 0, nkp = 0, nl = 0, nb = 0, B = 0;
	cudaStream_t st = nullptr;
	cudaEvent_t ev0 = nullptr, ev1 = nullptr;	// bracket the kernels of the last accumulate
	float last_ms = 0.f;
	int* ib = nullptr;
	double *b0 = nullptr, *br = nullptr, *j0 = nullptr, *jr = nullptr, *y0T = nullptr, *pm = nullptr;
	double *kr = nullptr, *coskt = nullptr, *sinkt = nullptr, *coskp = nullptr, *sinkp = nullptr;
	double2* e0 = nullptr;
	double2 *temp = nullptr, *temq = nullptr, *U = nullptr, *W = nullptr, *work = nullptr, *cbuf = nullptr;
	double *dclock = nullptr, *da1 = nullptr;
	std::vector<double> clock;	// [inst][4]: time, disx, disy, disz (host, updated in the reference's order)
	int* dact = nullptr;		// [inst]: takes the accumulate being enqueued (runs of the length-gauge engine)
};

namespace {

void pcs_free(qpc_pcs* h)
{
	if (!h) return;
	cudaSetDevice(h->dev);
	void* ps[] = {h->ijlT, h->plm, h->kr, h->exm, h->cps, h->cbuf, h->Q, h->out};
	for (void* p : ps) if (p) cudaFree(p);
	if (h->ev0) cudaEventDestroy(h->ev0);
	if (h->ev1) cudaEventDestroy(h->ev1);
	if (h->st) cudaStreamDestroy(h->st);
	delete h;
}

void ts_free(qpc_tsurff* h)
{
	if (!h) return;
	cudaSetDevice(h->dev);
	void* ps[] = {h->ib, h->b0, h->br, h->j0, h->jr, h->y0T, h->pm, h->kr, h->coskt, h->sinkt, h->coskp, h->sinkp, h->e0, h->temp, h->temq,
		h->U, h->W, h->work, h->cbuf, h->dclock, h->da1, h->dact};
	for (void* p : ps) if (p) cudaFree(p);
	if (h->ev0) cudaEventDestroy(h->ev0);
	if (h->ev1) cudaEventDestroy(h->ev1);
	if (h->st) cudaStreamDestroy(h->st);
	delete h;
}

template <class T> int grow(T** p, long* cap, long n)
{
	if (*cap >= n) return QPC_OK;
	if (*p) cudaFree(*p);
	*p = nullptr; *cap = 0;
	if (int rc = dalloc(p, (size_t)n)) return rc;
	*cap = n;
	return QPC_OK;
}

// PCS measurement on device wavefunctions c (host layout); writes the host output
int pcs_run(qpc_pcs* h, int kind, const double2* c, int n_inst, double* out)
{
	const qpc_dims& d = h->d;
	const int nch = d.n_m * d.n_l;
	if (int rc = grow(&h->Q, &h->cap_q, (long)n_inst * h->nkr * nch)) return rc;
	long total = kind == QPC_SPEC_LMD ? (long)n_inst * h->nkr * nch
		: kind == QPC_SPEC_PMD ? (long)n_inst * h->nkr * h->nkt * h->nkp : (long)n_inst * h->nkr * h->nkt;
	if (int rc = grow(&h->out, &h->cap_o, total)) return rc;
	dim3 g1((n_inst + PG - 1) / PG, (h->nkr + 127) / 128, nch);
	QPC_CUDA(cudaEventRecord(h->ev0, h->st));
	k_pcs_proj<<<g1, 128, 0, h->st>>>(h->ijlT, h->cps, c, h->Q, h->nkr, d.n_r, d.n_l, d.m0, nch, h->nl, n_inst);
	QPC_CUDA(cudaGetLastError());
	k_pcs_out<<<(unsigned)((total + 255) / 256), 256, 0, h->st>>>(kind, h->Q, h->plm, h->exm, h->kr, h->out, h->nkr, h->nkt, h->nkp,
		d.n_l, d.n_m, total);
	QPC_CUDA(cudaGetLastError());
	QPC_CUDA(cudaEventRecord(h->ev1, h->st));
	if (int rc = copy_to_host(out, h->out, sizeof(double2) * total, h->st)) return rc;
	QPC_CUDA(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
	return QPC_OK;
}

// one accumulate, enqueued on st without a wait: the surface values come from c (host layout
// [inst][m][l][r]) or, when eng != NULL, from the length-gauge engine's resident state (eng = the
// state, slot = the slot of each instance); act (host, may be NULL = every instance) selects the
// instances that take it.  The clock advances on the host in the reference's order.
int ts_enqueue(qpc_tsurff* h, int mode, const double* a, double dt, const double2* c, const double2* eng, const int* slot,
	const int* act, cudaStream_t st)
{
	const qpc_dims& d = h->d;
	const int B = h->B, nch = d.n_m * d.n_l;
	// the clock, as prepare(ax, ay, az, dt) advances it (momentum_1e.hpp:620-626)
	std::vector<double> a1((size_t)B * 2, 0.0);
	for (int i = 0; i < B; ++i) {
		if (act && !act[i]) continue;
		double* ck = &h->clock[4 * (size_t)i];
		double ax = 0.0, ay = 0.0, az = 0.0;
		if (mode == QPC_TSURFF_Z) { az = 0.5 * (a[2 * i] + a[2 * i + 1]); a1[i] = a[2 * i + 1]; }
		if (mode == QPC_TSURFF_XY) {
			ax = 0.5 * (a[4 * i] + a[4 * i + 1]); ay = 0.5 * (a[4 * i + 2] + a[4 * i + 3]);
			a1[2 * i] = a[4 * i + 1]; a1[2 * i + 1] = a[4 * i + 3];
		}
		ck[0] += dt; ck[1] += ax * dt; ck[2] += ay * dt; ck[3] += az * dt;
	}
	QPC_CUDA(cudaMemcpyAsync(h->dclock, h->clock.data(), sizeof(double) * 4 * B, cudaMemcpyHostToDevice, st));
	QPC_CUDA(cudaMemcpyAsync(h->da1, a1.data(), sizeof(double) * 2 * B, cudaMemcpyHostToDevice, st));
	if (act) QPC_CUDA(cudaMemcpyAsync(h->dact, act, sizeof(int) * B, cudaMemcpyHostToDevice, st));
	const long nsurf = (long)B * nch;
	if (eng) k_ts_prepare_eng<<<(unsigned)((nsurf + 255) / 256), 256, 0, st>>>(eng, slot, h->ib, h->b0, h->br, h->nb, d.n_m, d.n_r, d.n_l, nsurf,
		h->temp, h->temq);
	else k_ts_prepare<<<(unsigned)((nsurf + 255) / 256), 256, 0, st>>>(c, h->ib, h->b0, h->br, h->nb, d.n_r, nsurf, h->temp, h->temq);
	const long nu = (long)B * h->nkr * nch;
	k_ts_u<<<(unsigned)((nu + 255) / 256), 256, 0, st>>>(mode, h->temp, h->temq, h->j0, h->jr, h->pm, h->pm + nch, h->pm + 2 * nch, h->da1,
		h->nkr, d.n_l, d.n_m, d.m0, h->nl, nu, h->U);
	const int tw = h->nkt >= 128 ? 128 : 32 * ((h->nkt + 31) / 32);
	dim3 gw((h->nkt + tw - 1) / tw, h->nkr, B * d.n_m);
	k_ts_w<<<gw, tw, sizeof(double2) * d.n_l, st>>>(h->U, h->y0T, h->nkr, h->nkt, d.n_l, d.n_m, h->W);
	const long na = (long)B * h->nkr * h->nkt * h->nkp;
	k_ts_acc<<<(unsigned)((na + 255) / 256), 256, 0, st>>>(mode, h->W, h->e0, h->kr, h->coskt, h->sinkt, h->coskp, h->sinkp, h->dclock, dt,
		h->nkr, h->nkt, h->nkp, d.n_m, na, h->work, act ? h->dact : nullptr);
	QPC_CUDA(cudaGetLastError());
	return QPC_OK;
}

// one accumulate on device wavefunctions c (host layout), waited for
int ts_run(qpc_tsurff* h, int mode, const double* a, double dt, const double2* c)
{
	// the stream idle first (bounded): the copies from host memory never wait for queued work
	if (int rc = wait_on(h->st)) return rc;
	QPC_CUDA(cudaEventRecord(h->ev0, h->st));
	if (int rc = ts_enqueue(h, mode, a, dt, c, nullptr, nullptr, nullptr, h->st)) return rc;
	QPC_CUDA(cudaEventRecord(h->ev1, h->st));
	if (int rc = wait_on(h->st)) return rc;
	QPC_CUDA(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
	return QPC_OK;
}

}  // namespace

namespace qpc {
int tsurff_check_grid(qpc_tsurff* t, const qpc_dims& d)
{
	if (d.n_r != t->d.n_r || d.n_l != t->d.n_l || d.n_m != t->d.n_m || d.m0 != t->d.m0 || d.n_inst != t->B) {
		set_error("grid or batch of the t-SURFF handle differs from the propagator's"); return QPC_ERR_ARGS;
	}
	return QPC_OK;
}
int tsurff_enqueue_engine(qpc_tsurff* t, const void* st, const int* slot_dev, const double* a, const int* act, double dt, void* stream)
{
	return ts_enqueue(t, QPC_TSURFF_Z, a, dt, nullptr, (const double2*)st, slot_dev, act, (cudaStream_t)stream);
}
} // namespace qpc

extern "C" {

int qpc_pcs_create(const qpc_dims* dims, const qpc_kgrid* g, const double* kr, const double* ijl, const double* plm,
	const double* exm, const double* cps, qpc_pcs** out)
{
	if (!out) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	*out = nullptr;
	if (!grid_ok(dims, g) || !kr || !ijl || !plm || !exm || !cps) { set_error("bad arguments"); return QPC_ERR_ARGS; }
	if (dims->n_l * dims->n_m > 65535) { set_error("too many channels"); return QPC_ERR_ARGS; }
	int dev, rc;
	if ((rc = check_device(&dev))) return rc;
	qpc_pcs* h = new qpc_pcs;
	h->dev = dev; h->d = *dims; h->nkr = g->nkr; h->nkt = g->nkt; h->nkp = g->nkp; h->nl = lmax_of(*dims) + 1;
	auto fail = [&](int r) { pcs_free(h); return r; };
	if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&h->ev0) != cudaSuccess ||
		cudaEventCreate(&h->ev1) != cudaSuccess) { set_error("stream or event creation failed"); return fail(QPC_ERR_CUDA); }
	const int n = dims->n_r, nl = h->nl, nk = g->nkr, nch = dims->n_m * dims->n_l;
	std::vector<double> t((size_t)nl * n * nk);
	for (int k = 0; k < nk; ++k)
		for (int l = 0; l < nl; ++l)
			for (int r = 0; r < n; ++r) t[((size_t)l * n + r) * nk + k] = ijl[((size_t)k * nl + l) * n + r];
	if ((rc = upload(&h->ijlT, t.data(), t.size()))) return fail(rc);
	if ((rc = upload(&h->plm, plm, (size_t)g->nkt * nch))) return fail(rc);
	if ((rc = upload(&h->kr, kr, (size_t)nk))) return fail(rc);
	if ((rc = upload(&h->exm, (const double2*)exm, (size_t)g->nkp * dims->n_m))) return fail(rc);
	if ((rc = upload(&h->cps, (const double2*)cps, (size_t)nk * nl))) return fail(rc);
	*out = h;
	return QPC_OK;
}

int qpc_pcs_destroy(qpc_pcs* h)
{
	pcs_free(h);
	return QPC_OK;
}

int qpc_pcs_measure(qpc_pcs* h, int32_t kind, const double* coef, int32_t on_device, int32_t n_inst, double* out)
{
	if (!h || !coef || !out || n_inst < 1 || kind < QPC_SPEC_LMD || kind > QPC_SPEC_PAD) { set_error("bad arguments"); return QPC_ERR_ARGS; }
	if ((long)h->d.n_m * h->d.n_l > 65535 || (h->nkr + 127) / 128 > 65535) { set_error("too many channels or momenta for one launch"); return QPC_ERR_ARGS; }
	QPC_CUDA(cudaSetDevice(h->dev));
	const double2* c = (const double2*)coef;
	if (!on_device) {
		const long n = (long)n_inst * h->d.n_m * h->d.n_l * h->d.n_r;
		if (int rc = grow(&h->cbuf, &h->cap_c, n)) return rc;
		if (int rc = wait_on(h->st)) return rc;
		QPC_CUDA(cudaMemcpyAsync(h->cbuf, coef, sizeof(double2) * n, cudaMemcpyHostToDevice, h->st));
		c = h->cbuf;
	}
	return pcs_run(h, kind, c, n_inst, out);
}

int qpc_lgwz_pcs(qpc_lgwz* prop, qpc_pcs* h, int32_t kind, double* out)
{
	qpc_dims d;
	if (!prop || !h || !out) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	if (int rc = qpc_lgwz_dims(prop, &d)) return rc;
	if (d.n_r != h->d.n_r || d.n_l != h->d.n_l || d.n_m != h->d.n_m || d.m0 != h->d.m0) { set_error("grid of the propagator differs"); return QPC_ERR_ARGS; }
	QPC_CUDA(cudaSetDevice(h->dev));
	const long n = (long)d.n_inst * d.n_m * d.n_l * d.n_r;
	if (int rc = grow(&h->cbuf, &h->cap_c, n)) return rc;
	if (int rc = qpc_lgwz_get_device(prop, (double*)h->cbuf)) return rc;
	return qpc_pcs_measure(h, kind, (const double*)h->cbuf, 1, d.n_inst, out);
}

int qpc_tsurff_create(const qpc_dims* dims, const qpc_kgrid* g, const double* kr, const double* kt, const double* kp, int32_t nb,
	const int32_t* ib, const double* b0, const double* br, const double* j0, const double* jr, const double* y0, const double* e0,
	const double* pmat, qpc_tsurff** out)
{
	if (!out) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	*out = nullptr;
	if (!grid_ok(dims, g) || dims->n_inst < 1 || nb < 0 || nb > QPC_MAX_RANK + 1 || !kr || !kt || !kp || (nb && (!ib || !b0 || !br)) ||
		!j0 || !jr || !y0 || !e0 || !pmat) { set_error("bad arguments"); return QPC_ERR_ARGS; }
	for (int i = 0; i < nb; ++i) if (ib[i] < 0 || ib[i] >= dims->n_r) { set_error("ib[%d] = %d outside the grid", i, ib[i]); return QPC_ERR_ARGS; }
	if ((long)g->nkr * dims->n_inst * dims->n_m > 2147483647L || g->nkr > 65535 || (long)dims->n_inst * dims->n_m > 65535) {
		set_error("momentum grid or batch too large"); return QPC_ERR_ARGS;
	}
	int dev, rc;
	if ((rc = check_device(&dev))) return rc;
	qpc_tsurff* h = new qpc_tsurff;
	h->dev = dev; h->d = *dims; h->B = dims->n_inst; h->nkr = g->nkr; h->nkt = g->nkt; h->nkp = g->nkp; h->nb = nb; h->nl = lmax_of(*dims) + 1;
	auto fail = [&](int r) { ts_free(h); return r; };
	if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&h->ev0) != cudaSuccess ||
		cudaEventCreate(&h->ev1) != cudaSuccess) { set_error("stream or event creation failed"); return fail(QPC_ERR_CUDA); }
	const int nch = dims->n_m * dims->n_l, B = h->B;
	std::vector<int> ibv(ib, ib + nb);
	if ((rc = upload(&h->ib, nb ? ibv.data() : nullptr, nb))) return fail(rc);
	if ((rc = upload(&h->b0, b0, nb)) || (rc = upload(&h->br, br, nb))) return fail(rc);
	if ((rc = upload(&h->j0, j0, (size_t)g->nkr * h->nl)) || (rc = upload(&h->jr, jr, (size_t)g->nkr * h->nl))) return fail(rc);
	std::vector<double> yT((size_t)nch * g->nkt);
	for (int t = 0; t < g->nkt; ++t)
		for (int c = 0; c < nch; ++c) yT[(size_t)c * g->nkt + t] = y0[(size_t)t * nch + c];
	if ((rc = upload(&h->y0T, yT.data(), yT.size()))) return fail(rc);
	if ((rc = upload(&h->pm, pmat, (size_t)3 * nch))) return fail(rc);
	if ((rc = upload(&h->e0, (const double2*)e0, (size_t)g->nkp * dims->n_m))) return fail(rc);
	std::vector<double> ct(g->nkt), st(g->nkt), cp(g->nkp), sp(g->nkp);
	for (int i = 0; i < g->nkt; ++i) { ct[i] = std::cos(kt[i]); st[i] = std::sin(kt[i]); }
	for (int i = 0; i < g->nkp; ++i) { cp[i] = std::cos(kp[i]); sp[i] = std::sin(kp[i]); }
	if ((rc = upload(&h->kr, kr, g->nkr)) || (rc = upload(&h->coskt, ct.data(), ct.size())) || (rc = upload(&h->sinkt, st.data(), st.size())) ||
		(rc = upload(&h->coskp, cp.data(), cp.size())) || (rc = upload(&h->sinkp, sp.data(), sp.size())))
		return fail(rc);
	if ((rc = dalloc(&h->temp, (size_t)B * nch)) || (rc = dalloc(&h->temq, (size_t)B * nch)) ||
		(rc = dalloc(&h->U, (size_t)B * g->nkr * nch)) || (rc = dalloc(&h->W, (size_t)B * g->nkr * g->nkt * dims->n_m)) ||
		(rc = dalloc(&h->work, (size_t)B * g->nkr * g->nkt * g->nkp)) || (rc = dalloc(&h->cbuf, (size_t)B * nch * dims->n_r)) ||
		(rc = dalloc(&h->dclock, (size_t)4 * B)) || (rc = dalloc(&h->da1, (size_t)2 * B)) || (rc = dalloc(&h->dact, (size_t)B)))
		return fail(rc);
	h->clock.assign((size_t)4 * B, 0.0);
	if (cudaMemset(h->work, 0, sizeof(double2) * (size_t)B * g->nkr * g->nkt * g->nkp) != cudaSuccess) { set_error("cudaMemset failed"); return fail(QPC_ERR_CUDA); }
	*out = h;
	return QPC_OK;
}

int qpc_tsurff_destroy(qpc_tsurff* h)
{
	ts_free(h);
	return QPC_OK;
}

int qpc_tsurff_clear(qpc_tsurff* h)
{
	if (!h) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	QPC_CUDA(cudaSetDevice(h->dev));
	std::fill(h->clock.begin(), h->clock.end(), 0.0);
	QPC_CUDA(cudaMemsetAsync(h->work, 0, sizeof(double2) * (size_t)h->B * h->nkr * h->nkt * h->nkp, h->st));
	return wait_on(h->st);
}

int qpc_tsurff_accumulate(qpc_tsurff* h, int32_t mode, const double* a, double dt, const double* coef, int32_t on_device)
{
	if (!h || !coef || mode < QPC_TSURFF_FREE || mode > QPC_TSURFF_XY || (mode != QPC_TSURFF_FREE && !a) || !std::isfinite(dt)) {
		set_error("bad arguments"); return QPC_ERR_ARGS;
	}
	QPC_CUDA(cudaSetDevice(h->dev));
	const double2* c = (const double2*)coef;
	if (!on_device) {
		const long n = (long)h->B * h->d.n_m * h->d.n_l * h->d.n_r;
		if (int rc = wait_on(h->st)) return rc;
		QPC_CUDA(cudaMemcpyAsync(h->cbuf, coef, sizeof(double2) * n, cudaMemcpyHostToDevice, h->st));
		c = h->cbuf;
	}
	return ts_run(h, mode, a, dt, c);
}


int qpc_lgwz_tsurff(qpc_lgwz* prop, qpc_tsurff* h, int32_t mode, const double* a, double dt)
{
	qpc_dims d;
	if (!prop || !h) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	if (int rc = qpc_lgwz_dims(prop, &d)) return rc;
	if (d.n_r != h->d.n_r || d.n_l != h->d.n_l || d.n_m != h->d.n_m || d.m0 != h->d.m0 || d.n_inst != h->B) {
		set_error("grid or batch of the propagator differs"); return QPC_ERR_ARGS;
	}
	QPC_CUDA(cudaSetDevice(h->dev));
	if (int rc = qpc_lgwz_get_device(prop, (double*)h->cbuf)) return rc;
	return qpc_tsurff_accumulate(h, mode, a, dt, (const double*)h->cbuf, 1);
}

int qpc_vgwr_tsurff(qpc_vgwr* prop, qpc_tsurff* h, int32_t mode, const double* a, double dt)
{
	qpc_dims d;
	if (!prop || !h) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	if (int rc = qpc_vgwr_dims(prop, &d)) return rc;
	if (d.n_r != h->d.n_r || d.n_l != h->d.n_l || d.n_m != h->d.n_m || d.m0 != h->d.m0 || d.n_inst != h->B) {
		set_error("grid or batch of the propagator differs"); return QPC_ERR_ARGS;
	}
	QPC_CUDA(cudaSetDevice(h->dev));
	if (int rc = qpc_vgwr_get_device(prop, (double*)h->cbuf)) return rc;
	return qpc_tsurff_accumulate(h, mode, a, dt, (const double*)h->cbuf, 1);
}

int qpc_pcs_last_run(qpc_pcs* h, float* ms)
{
	if (!h || !ms) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	*ms = h->last_ms;
	return QPC_OK;
}

int qpc_tsurff_last_run(qpc_tsurff* h, float* ms)
{
	if (!h || !ms) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	*ms = h->last_ms;
	return QPC_OK;
}

int qpc_tsurff_get(qpc_tsurff* h, double* work, double* clock)
{
	if (!h || !work) { set_error("NULL argument"); return QPC_ERR_ARGS; }
	QPC_CUDA(cudaSetDevice(h->dev));
	if (int rc = copy_to_host(work, h->work, sizeof(double2) * (size_t)h->B * h->nkr * h->nkt * h->nkp, h->st)) return rc;
	if (clock) std::copy(h->clock.begin(), h->clock.end(), clock);
	return QPC_OK;
}

}  // extern "C"
