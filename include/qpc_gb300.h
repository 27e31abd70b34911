/*
 * qpc_gb300.h -- C ABI of the GB300 propagation engine for QPC-TDSE.
 *
 * The reference (zzh535897/QPC-TDSE-CPC) has no runtime plugin API: its
 * propagators are C++ templates selected at compile time
 * (binsrc/sphTDSE.cpp:574-600) and called from the driver's step loop
 * (binsrc/sphTDSE.cpp:786-831).  This header is the boundary a caller crosses
 * instead: plain C types, host pointers, int status codes, no C++ exceptions
 * and no torch types.  Each entry point names the reference member it replaces.
 *
 * Layouts (identical to the reference, so state export is a memcpy):
 *   wavefunction  c[inst][m][l][r] complex128 (re, im interleaved)
 *                 (spherical/coefficient/1e.hpp, recvec<comp_t,recidx<m,l,r>>)
 *   radial band   A[r*(p+1)+k] = A(r, r+k), k = 0..p, real float64
 *                 (spherical/operators/1e.hpp:20)
 *   H per l       H[l][r][k] for l = 0..lmax, lmax = max|m| + n_l - 1
 *                 (spherical/operators/1e.hpp:595-648)
 *
 * Status codes: 0 on success, a QPC_ERR_* value otherwise; qpc_last_error()
 * returns a message for the calling thread's last failure.  Nothing here
 * throws, aborts, traps a GPU or waits without a bound.
 */
#ifndef QPC_GB300_H
#define QPC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QPC_OK 0
#define QPC_ERR_ARGS 1      /* bad dimensions, pointers or values */
#define QPC_ERR_NOMEM 2     /* device or host allocation failed */
#define QPC_ERR_CUDA 3      /* a CUDA call failed */
#define QPC_ERR_SINGULAR 4  /* a zero pivot in a factorisation */
#define QPC_ERR_NUMERIC 5   /* non-finite value or no convergence */
#define QPC_ERR_TIMEOUT 6   /* a bounded wait for the device ran out */
#define QPC_ERR_STATE 7     /* call made in the wrong state */
#define QPC_ERR_NODEVICE 8  /* no CUDA device, or not a GB300-class device */

#define QPC_MAX_RANK 8      /* largest B-spline degree p the engine accepts */

enum { QPC_POTENTIAL_HYDROGENIC = 0, QPC_POTENTIAL_YUKAWA = 1 };

/* V(r) = -zc/r (hydrogenic, spherical/potential.hpp:9-17) or
 * V(r) = -(zc + zs exp(-sigma r))/r (hydrogenic_yukawa, potential.hpp:19-29). */
typedef struct qpc_potential {
	int32_t kind;
	double zc, zs, sigma;
} qpc_potential;

/* Grid of one batch; replaces dimension_1e<nr,mr,nl,nm,m0> (spherical/dimension/1e.hpp:20-127). */
typedef struct qpc_dims {
	int32_t n_r;    /* active radial B-splines   (dims_t::n_dims) */
	int32_t p;      /* B-spline degree            (dims_t::n_diag); bands hold p+1 per row */
	int32_t n_l;    /* l channels per m           (dims_t::l_dims); l = |m| + il */
	int32_t n_m;    /* m channels                 (dims_t::m_dims) */
	int32_t m0;     /* first m                    (dims_t::m_init) */
	int32_t n_inst; /* wavefunctions advanced together (1 for the plain path) */
} qpc_dims;

const char* qpc_last_error(void);
/* Engine version string; also reports the SM arch the library was built for. */
const char* qpc_version(void);

/* Bound, in seconds, of every wait of this library's host code for the GPU (process-wide;
 * default 600 s, or the value of the environment variable QPC_WAIT_LIMIT_S when it is set
 * before the first wait).  A wait that runs out returns QPC_ERR_TIMEOUT; the work it waited
 * for stays queued on the handle's stream and the next call on the handle waits for it
 * again.  Results reach host memory only after a wait has succeeded, so a call that times
 * out leaves no copy pending into the caller's buffers.  The reference's calls have no such
 * channel: they run on the calling host thread (its propagate is noexcept, cn_1e.hpp:595).
 * Errors: QPC_ERR_ARGS for a value that is not positive and finite. */
int qpc_set_wait_limit(double seconds);
double qpc_get_wait_limit(void);

/* FP64 FMA throughput of the current device in TFLOP/s (FMA = 2 flops), measured by a probe
 * kernel of independent DFMA chains timed with CUDA events (best of 5 launches of ~20 ms):
 * the denominator of the FP64 roofline fractions this engine reports.  No counterpart in the
 * reference. */
int qpc_fp64_peak(double* tflops);

/* ---------------------------------------------------------------- setup (host)
 * One-time matrix construction, done on the host as in the reference. */

/* Knots of bsplines::initialize_axis_linear_step (functions/basis_bsplines.h:450-459):
 * writes n_r + p + 3 values. */
int qpc_linear_knots(int32_t n_r, int32_t p, double rmin, double rmax, double* knots);

/* integrator_radi::integrate_0r0 / _0r1 / integrate_hc (spherical/utilities/basisfunc.hpp:63-106)
 * on the given knots with 2p+2 Gauss-Legendre points per interval:
 * S = <Bi|Bj>, R = <Bi|r|Bj>, Rinv = <Bi|1/r|Bj>, D = <Bi|d/dr Bj>,
 * H[l] = <Bi|V + l(l+1)/(2 mass r^2)|Bj> + <Bi'|Bj'>/(2 mass) for l < n_lh.
 * Any output pointer may be NULL. */
int qpc_radial_setup(int32_t n_r, int32_t p, int32_t n_lh, const double* knots, const qpc_potential* pot,
	double mass, double* S, double* R, double* Rinv, double* D, double* H);

/* integrator_angu::integrate_cos (spherical/utilities/basisfunc.hpp:222-229): y10[il] = <l,m|cos|l+1,m>. */
int qpc_y10_coupling(int32_t n_l, int32_t m, double* y10);

/* operator_y10::solve_eigen for one m (spherical/operators/1e.hpp:304-333):
 * lam[n_l] ascending, P[n_l][n_l] row-major with row a = eigenvector a. */
int qpc_y10_eigen(int32_t n_l, int32_t m, double* lam, double* P);

/* lu_zsb of S + i g H (algorithm/ed.h:208-289) in the engine's layout:
 * Lrow[r][k-1] = L(r, r-k) (complex), Dinv[r] = 1/D(r) (complex).
 * Returns the count of pivots with |D|^2 < 1e-31, or -1 on bad arguments. */
int qpc_ldlt_csym(int32_t n, int32_t p, const double* S, const double* H, double g, double* Lrow, double* Dinv);

/* gv_dsb (LAPACKE_dsbgv, algorithm/ed.h:105-112): all eigenvalues of H v = E S v
 * ascending, and the lowest n_want S-normalised eigenvectors (rows of vec). */
int qpc_gen_eigen(int32_t n, int32_t p, const double* S, const double* Hl, int32_t n_want, double* energy, double* vec);

/* Angular couplings of propagator_cn_hc_vgwr (cn_1e.hpp:836-890) on the channels
 * ch = im*n_l + il: comp 0 = x1 (Y11, mult 1), 1 = x2 (Q11, mult -i), 2 = y1 (Y11, mult -i),
 * 3 = y2 (Q11, mult 1) (operator_y11/q11::solve_eigen, operators/1e.hpp:336-523).
 * lam[N_ch] ascending and P[N_ch][N_ch] complex with P Z P^H = diag(lam). */
int qpc_vgwr_angular(int32_t n_l, int32_t n_m, int32_t m0, int32_t comp, double* lam, double* P);

/* absorber_mask::initialize (absorber.hpp:42-49): M[r][k] = <B_r| m |B_{r+k}> with
 * m(r) = 1 below rmin, 0 above rmax, |cos(pi/2 (r-rmin)/(rmax-rmin))|^index between
 * (the reference's default index is 1/6). */
int qpc_mask_band(int32_t n_r, int32_t p, const double* knots, double rmin, double rmax, double index, double* M);

/* lu_dsb (LAPACKE_dpbtrf 'L', algorithm/ed.h:182-193) as operator_sc::initialize uses it
 * (spherical/operators/1e.hpp:1233-1244): S = L L^T with L(r+k, r) at L[r*(p+1)+k], the
 * layout of operator_sc::cholesky(); entries past the last row are zero.  Returns 0, -1 on
 * bad arguments, or 1 + the row of the first non-positive pivot. */
int qpc_cholesky_band(int32_t n, int32_t p, const double* S, double* L);

/* field_component_sinen<n_pow> inside field<> (structure/field.h:89-133, 245-281):
 * *nt_out = para_nt; when f != NULL writes f(t_i), i = 0..para_nt (cap >= para_nt+1). */
int qpc_field_sinen(int32_t n_pow, double e0, double w0, double nc, double n0, double cep, double dt,
	int64_t cap, double* f, int64_t* nt_out);

/* ---------------------------------------------------------------- propagator
 * propagator_cn_hc_lgwz (spherical/propagator/cn_1e.hpp:549-619): length gauge,
 * field along z, Crank-Nicolson split operator, for a batch of n_inst
 * wavefunctions that share one grid, potential and dt.  The handle owns its
 * device memory and one CUDA stream; calls on one handle are not re-entrant,
 * calls on different handles may come from different threads. */
typedef struct qpc_lgwz qpc_lgwz;

/* Replaces propagator_cn_hc_lgwz::initialize(nthd, radi, angu, mass, potn, dt)
 * (cn_1e.hpp:565-593).  S, R: [n_r][p+1]; H: [lmax+1][n_r][p+1] with
 * lmax = max(|m0|, |m0+n_m-1|) + n_l - 1.  Builds the field-free bands and
 * their LDL^T (cn_component_hc::initialize) and the Y10 eigensystem per m.
 * Errors: QPC_ERR_ARGS, QPC_ERR_NODEVICE, QPC_ERR_NOMEM, QPC_ERR_SINGULAR. */
int qpc_lgwz_create(const qpc_dims* dims, double dt, const double* S, const double* R, const double* H, qpc_lgwz** out);

/* The same with one potential per wavefunction when h_per_instance != 0: H is then
 * [n_inst][lmax+1][n_r][p+1] and each instance gets its own field-free factorisation (the
 * coupling step depends only on S and R, which the batch shares).  For batches that share a
 * grid but not a potential, such as the screened-Coulomb atoms of a mixed batch
 * (spherical/potential.hpp:19-29); the reference builds one propagator per potential. */
int qpc_lgwz_create_ex(const qpc_dims* dims, double dt, const double* S, const double* R, const double* H, int32_t h_per_instance,
	qpc_lgwz** out);

/* Frees everything the handle owns.  NULL is accepted. */
int qpc_lgwz_destroy(qpc_lgwz* h);

/* Copy the batch state in/out, host layout c[inst][m][l][r] complex128
 * (what coefficient<dims_t>::data holds, coefficient/1e.hpp:11-53). */
int qpc_lgwz_put(qpc_lgwz* h, const double* coef);
int qpc_lgwz_get(qpc_lgwz* h, double* coef);
/* Same, with device-resident buffers in the host layout (no host copy). */
int qpc_lgwz_put_device(qpc_lgwz* h, const double* dev_coef);
int qpc_lgwz_get_device(qpc_lgwz* h, double* dev_coef);
/* The grid and batch size the handle was created with. */
int qpc_lgwz_dims(qpc_lgwz* h, qpc_dims* dims);
/* The handle's CUDA stream (a cudaStream_t): every call on the handle is ordered on it,
 * so a caller can order its own device work (events, copies into put_device buffers)
 * before or after the engine's.  No counterpart in the reference (it has no device code). */
int qpc_lgwz_stream(qpc_lgwz* h, void** stream);

/* One call of propagate(coef, ez_ti, ez_tf) (cn_1e.hpp:595-613) for every
 * instance: f_ti[inst], f_tf[inst] are the field at t_i and t_{i+1}. */
int qpc_lgwz_propagate(qpc_lgwz* h, const double* f_ti, const double* f_tf);

/* One field-free propagate(coef) (cn_1e.hpp:615-618) for every instance. */
int qpc_lgwz_propagate_free(qpc_lgwz* h);

/* The driver loop (binsrc/sphTDSE.cpp:786-831) for the whole batch in one call:
 * instance k takes nt_field[k] field steps with f(t_i) = ftab[k*ld + i],
 * i = 0..nt_field[k] (nt_field[k]+1 values), then field-free steps until
 * nt_total[k] >= nt_field[k] steps in all.  Instances advance independently,
 * so uneven step counts are fine.  The result equals nt_total[k] single calls
 * (within rounding: consecutive coupling half-steps are fused). */
int qpc_lgwz_run(qpc_lgwz* h, const double* ftab, int64_t ld, const int64_t* nt_field, const int64_t* nt_total);
/* qpc_lgwz_run on n distinct handles at once, each from its own host thread on its
 * own streams: handle i takes (ftab[i], ld[i], nt_field[i], nt_total[i]).  For
 * batches on different grids (the driver loop of sphTDSE.cpp:786-831 for several
 * dimension_1e instantiations side by side).  Returns the first failing handle's
 * status (its index in *failed when failed != NULL, else -1). */
int qpc_lgwz_run_many(int32_t n, qpc_lgwz* const* hs, const double* const* ftab, const int64_t* ld,
	const int64_t* const* nt_field, const int64_t* const* nt_total, int32_t* failed);

/* qpc_lgwz_run that also records, for every instance k and step s < nt_total[k],
 * zlist[k*ldz + s] = Re <psi_k(t_s)| f(r) cos(theta) |psi_k(t_s)> with F = <Bi|f|Bj>
 * ([n_r][p+1]; f(r) = r gives the dipole), the observation the driver makes before
 * each step (obsv::observe, binsrc/sphTDSE.cpp:515-521 and 794).  ldz >= max nt_total. */
int qpc_lgwz_run_dipole(qpc_lgwz* h, const double* ftab, int64_t ld, const int64_t* nt_field, const int64_t* nt_total,
	const double* F, double* zlist, int64_t ldz);

/* What the driver loop does to the state after every propagate besides observing
 * (binsrc/sphTDSE.cpp:797-810): the t-SURFF accumulate (spec::accumulate with f(t_i), f(t_i+1)
 * during the pulse, the field-free accumulate after it) and then the absorbing mask
 * (absorber_mask::operator(), absorber.hpp:51-63).  Either may be NULL. */
typedef struct qpc_run_opts {
	const double* mask;             /* absorber band [n_r][p+1] (qpc_mask_band), or NULL */
	struct qpc_tsurff* tsurff;      /* t-SURFF handle over the same grid and batch (dt = the propagator's), or NULL */
} qpc_run_opts;
/* qpc_lgwz_run with the per-step t-SURFF accumulate and mask of opts applied to every
 * instance after each of its steps, on the device, without a host round trip: each coupling
 * step is then applied as its closing and opening halves around them.  Not combined with the
 * in-loop dipole (QPC_ERR_ARGS). */
int qpc_lgwz_run_ex(qpc_lgwz* h, const double* ftab, int64_t ld, const int64_t* nt_field, const int64_t* nt_total,
	const qpc_run_opts* opts);

/* S-norm per instance, sum over (m,l) of c^H S c
 * (operator_rsym::observe, spherical/operators/1e.hpp:69-89); norm[n_inst]. */
int qpc_lgwz_norm(qpc_lgwz* h, double* norm);
/* absorber_mask::operator()(coef, prop.s) (absorber.hpp:51-63) on every wavefunction of the
 * batch: c <- S^-1 (M c) per (m,l) channel, M from qpc_mask_band.  The driver loop applies it
 * after each propagate (sphTDSE.cpp:807-810). */
int qpc_lgwz_mask(qpc_lgwz* h, const double* M);

/* <c| f(r) cos(theta) |c> per instance with F = <Bi|f|Bj> ([n_r][p+1])
 * (observable_z::observe, spherical/observable/1e.hpp:26-50); out[2*inst] re, [2*inst+1] im. */
int qpc_lgwz_dipole(qpc_lgwz* h, const double* F, double* out);

/* eigenstate_sph::projection (spherical/spectrum/population_1e.hpp:29-55):
 * proj[inst][m][il][n] = sum_r basis_l[n][r] c[inst][m][il][r] for the
 * n_state[l] left eigenvectors (S v) of each l = 0..lmax, packed one l after
 * another in basis (n_state[l] rows of n_r each); proj is packed the same way
 * per (inst, m, il) with n_state[l] entries, complex. */
int qpc_lgwz_projection(qpc_lgwz* h, const int32_t* n_state, const double* basis, double* proj);

/* ---------------------------------------------------------------- spectra (host)
 * Harmonic spectrum of one wavefunction from its per-step dipole z(t_i), t_i = t0 + i dt
 * (the reference's analysis/plot_hhs.m): D(w) = DFT(-z window) dt/2pi with a sin^2
 * window on (tmin, tmax), S(w) = 4 pi^2 w^{+2 | -2} |D|^2 / c^2 (dipole_type 1 | 2),
 * w_k = 2 pi k/(n dt), k < ceil(n/2) values written to omega and spectrum. */
int qpc_hhg_spectrum(const double* z, int64_t n, double t0, double dt, double tmin, double tmax, int32_t dipole_type,
	double* omega, double* spectrum);

/* qpc_hhg_spectrum for n_inst dipole lists at once, on the GPU (the spectrum reduction of a
 * batched run): list i is z[i*ldz + j], j < n[i], t_j = t0 + j dt, windowed on (tmin[i], tmax[i]);
 * spectrum[i*kmax + k] = S(w_k) at w_k = 2 pi k / (n[i] dt) for k < kmax (0 for k >= ceil(n[i]/2)).
 * A direct DFT of the first kmax frequencies (those up to the harmonic orders of interest), not
 * an FFT of all n/2.  Same arguments and results as qpc_hhg_spectrum to rounding. */
int qpc_hhg_spectra(int32_t n_inst, const double* z, int64_t ldz, const int64_t* n, double t0, double dt, const double* tmin,
	const double* tmax, int32_t dipole_type, int64_t kmax, double* spectrum);

/* C = A B in FP64 on the bf16 tensor cores by exact digit slices (the product the velocity-gauge
 * transforms use): A [n][K] (row stride lda), B [K][M] (ldb), C [n][M] (ldc), host buffers.  Each
 * row of A and column of B is cut into 9 digits of 7 bits under the power of two of its largest
 * element; the digit products are summed exactly (fp32 tensor accumulation of integers below 2^24,
 * int64 across chunks) and rounded to FP64 once.  The error is near K 2^(ea_i + eb_j - 61), with
 * 2^ea_i and 2^eb_j the row's and column's powers of two: below an FP64 GEMM's own rounding.
 * ms (optional): device time of splitting B and the product. */
int qpc_dgemm_slices(int64_t n, int64_t M, int64_t K, const double* A, int64_t lda, const double* B, int64_t ldb, double* C,
	int64_t ldc, float* ms);

/* The length-gauge l-space transform of the coupling step, the engine's form of cn_transform_hl
 * (spherical/propagator/cn_1e.hpp:101-147), on the tensor cores as the engine runs it for
 * n_l <= 48: in and out are n_pos rows of n_l complex channel values (interleaved re, im; host
 * buffers); V [n_l/2 + 1][n_l] holds the eigenvectors of +s_k (rows k < n_l/2) and, for odd n_l, the
 * zero-eigenvalue vector (last row).  forward != 0: slot 2k = E_k + O_k, slot 2k+1 = conj(E_k - O_k)
 * and, for odd n_l, slot n_l - 1 = Z, with E_k, Z the sums over even l and O_k over odd l of V[k][l] c_l;
 * forward = 0: c_l = sum_k V[k][l] x_(2k + l%2) (with Z's row for even l).  The products are formed
 * in exact 8-bit digits (each row of real or imaginary parts under its power of two) and rounded
 * once: each E_k, O_k is within about n_l 2^(e + f - 59) of the exact sum, 2^e and 2^f the powers of
 * two of the input row and of V's row (an FP64 dot product rounds near n_l 2^(e + f - 53)).
 * Errors: QPC_ERR_ARGS (n_pos < 1, n_l outside 1..48, NULL buffers), QPC_ERR_TIMEOUT. */
int qpc_lspace_transform(int64_t n_pos, int32_t n_l, const double* V, int32_t forward, const double* in, double* out);

/* Photoelectron energy spectrum (|proj|^2 binned over [emin, emax) per unit energy) and
 * ionization yield 1 - sum_{energy < thres} |proj|^2 (ionization_sph::measure_ioyd,
 * spectrum/ionization_1e.hpp:15-51) from n projections (complex) with their energies. */
int qpc_pes_bin(const double* proj, const double* energy, int64_t n, double emin, double emax, int32_t nbins, double thres,
	double* pes, double* bound, double* yield);

/* Time the handle's last qpc_lgwz_run on its stream, in milliseconds
 * (CUDA events around the launched kernels). */
int qpc_lgwz_last_run_ms(qpc_lgwz* h, double* ms);

/* Kernel launches made by the handle since creation (all of them this library's own). */
int64_t qpc_lgwz_launch_count(qpc_lgwz* h);

/* Per-kernel timing of qpc_lgwz_run: when on, each launch is bracketed by CUDA
 * events on the handle's stream and run() accumulates the elapsed times per
 * kernel (setting it also clears the totals).  ms[QPC_NKERNEL], launches[QPC_NKERNEL]
 * are indexed by QPC_KERNEL_*. */
enum { QPC_KERNEL_FACTOR = 0, QPC_KERNEL_TRANSFORM_FWD = 1, QPC_KERNEL_SWEEP = 2,
       QPC_KERNEL_TRANSFORM_BWD = 3, QPC_KERNEL_FIELDFREE = 4, QPC_NKERNEL = 5 };
int qpc_lgwz_set_profiling(qpc_lgwz* h, int on);

/* Tuning state: out[0] = factorisation look-ahead (steps); out[1+b], out[33+b] =
 * lanes per real/imaginary part chosen by the autotuner for the coupling and the
 * field-free chain kernels at live-instance bucket b (2^(b-1) < live <= 2^b; 0 = not tuned yet).
 * out must hold 65 values. */
int qpc_lgwz_get_tuning(qpc_lgwz* h, int32_t* out);
int qpc_lgwz_kernel_times(qpc_lgwz* h, double* ms, int64_t* launches);

/* ---------------------------------------------------------------- velocity gauge, elliptical
 * Replaces propagator_cn_hc_vgwr (spherical/propagator/cn_1e.hpp:812-951): initialize with
 * S, Rinv = <B|1/r|B>, D = <B_i|d/dr B_j> (upper entries of the anti-symmetric band) and H
 * [lmax+1][n_r][p+1]; propagate(coef, ax_ti, ax_tf, ay_ti, ay_tf) and propagate(coef)
 * (cn_1e.hpp:903-950) per instance; run() the driver loop (sphTDSE.cpp:930-950 for the
 * elliptical pulse) with atab[inst][s][2] = (A_x, A_y)(t_s), s = 0..nt_field[inst].
 * The coupling transforms are dense n_m n_l x n_m n_l matrices, block-diagonal in l-parity,
 * applied by this library's own FP64 GEMM kernels. */
typedef struct qpc_vgwr qpc_vgwr;
int qpc_vgwr_create(const qpc_dims* dims, double dt, const double* S, const double* Rinv, const double* D, const double* H,
	qpc_vgwr** out);
int qpc_vgwr_destroy(qpc_vgwr* h);
int qpc_vgwr_put(qpc_vgwr* h, const double* coef);
int qpc_vgwr_get(qpc_vgwr* h, double* coef);
int qpc_vgwr_put_device(qpc_vgwr* h, const double* dev_coef);
int qpc_vgwr_get_device(qpc_vgwr* h, double* dev_coef);
int qpc_vgwr_dims(qpc_vgwr* h, qpc_dims* dims);
int qpc_vgwr_propagate(qpc_vgwr* h, const double* ax_ti, const double* ax_tf, const double* ay_ti, const double* ay_tf);
int qpc_vgwr_propagate_free(qpc_vgwr* h);
int qpc_vgwr_run(qpc_vgwr* h, const double* atab, int64_t ld, const int64_t* nt_field, const int64_t* nt_total);
/* qpc_vgwr_run that also records, for every instance k and step s < nt_total[k], the dipole
 * xlist[k*ldz + s] = <x>, ylist[k*ldz + s] = <y> of psi_k(t_s) with f(r) = r: F = <Bi|f|Bj>
 * ([n_r][p+1]), the observation the elliptical driver makes before each step (observable_r,
 * spherical/observable/1e.hpp:52-129: x = Re(rm + rp)/2, y = Im(rp - rm)/2; recorded at
 * binsrc/sphTDSE.cpp:515-527 and 933-934).  ldz >= max nt_total. */
int qpc_vgwr_run_dipole(qpc_vgwr* h, const double* atab, int64_t ld, const int64_t* nt_field, const int64_t* nt_total,
	const double* F, double* xlist, double* ylist, int64_t ldz);
int qpc_vgwr_norm(qpc_vgwr* h, double* norm);
int qpc_vgwr_last_run(qpc_vgwr* h, float* ms, int64_t* launches);
/* Per-kernel timing of qpc_vgwr_run: when on, each launch group is bracketed by CUDA events on
 * the handle's stream and run() accumulates the times per kind (setting it clears the totals):
 * ms[3], launches[3] for 0 = the (m,l) transforms (one entry per transform, both parity
 * blocks), 1 = the coupling Crank-Nicolson solves, 2 = the field-free step. */
int qpc_vgwr_set_profiling(qpc_vgwr* h, int on);
int qpc_vgwr_kernel_times(qpc_vgwr* h, double* ms, int64_t* launches);

/* ---------------------------------------------------------------- Arnoldi propagator
 * Replaces propagator_hc_lgwz (spherical/propagator/la_1e.hpp:390-444) with
 * propagate<1>(coef, dt) = propagator_arnoldi::propagate1 (la_1e.hpp:312-335):
 * per step w -> exp(-i dt S^-1 H) w in the Krylov space of S^-1 H built in the
 * S metric, H = H_l + ez R Y10, at most kmax vectors, expansion stopped when
 * <v|S|v> < 1e-13 (la_1e.hpp:223).  ez is the field member of the reference
 * class (la_1e.hpp:401), here given per instance and step.  S^-1 is the
 * per-(m,l)-channel Cholesky solve that operator_sc::inverse_sub performs
 * (operators/1e.hpp:1247-1251); the shipped operator_sc::inverse_all
 * (operators/1e.hpp:1253-1260) offsets channel i by i*n_r while stepping i by
 * n_r and so does not apply S^-1 to the (m,l) channels.
 * A handle holds n_inst wavefunctions on one radial grid and runs them as one
 * batch on its own CUDA stream; calls on different handles are independent.
 *   S, R   [n_r][p+1] overlap and <B|r|B> bands
 *   H      [h_per_instance ? n_inst : 1][lmax+1][n_r][p+1], lmax = max|m| + n_l - 1
 *          (operator_hc, operators/1e.hpp:595-648); per instance allows one
 *          potential per wavefunction on a shared grid
 *   y10    [n_m][n_l] <l,m|cos|l+1,m> (operator_y10, qpc_y10_coupling per m)
 *   emin, emax  the criterion thresholds (arnoldi_workspace, la_1e.hpp:54-62) */
typedef struct qpc_arnoldi qpc_arnoldi;
int qpc_arnoldi_create(const qpc_dims* dims, const double* S, const double* R, const double* H, int32_t h_per_instance,
	const double* y10, double dt, int32_t kmax, double emin, double emax, qpc_arnoldi** out);
int qpc_arnoldi_destroy(qpc_arnoldi* h);
/* state transfer, [n_inst][n_m][n_l][n_r] complex128, host or device pointers */
int qpc_arnoldi_put(qpc_arnoldi* h, const double* coef);
int qpc_arnoldi_get(qpc_arnoldi* h, double* coef);
int qpc_arnoldi_put_device(qpc_arnoldi* h, const double* dev_coef);
int qpc_arnoldi_get_device(qpc_arnoldi* h, double* dev_coef);
/* nt[k] steps of instance k with ez = ez[k*ld + s] during step s (nt[k] <= ld).  crit
 * and msub (either may be NULL) receive, at [k*ld + s], criterion() (la_1e.hpp:296-310:
 * 0 when |x_{m-1}|^2 > emax, 1 when > emin, else 2) and the Krylov dimension m of each
 * step; -1 for steps an instance does not take. */
int qpc_arnoldi_run(qpc_arnoldi* h, const double* ez, int64_t ld, const int64_t* nt, int8_t* crit, int8_t* msub);
/* one step of every instance with ez[k]; crit[k] as above (may be NULL) */
int qpc_arnoldi_propagate(qpc_arnoldi* h, const double* ez, int8_t* crit);
/* S-norm per instance (operator_sc::observe, operators/1e.hpp:69-79) */
int qpc_arnoldi_norm(qpc_arnoldi* h, double* norm);
/* device time of the last run (CUDA events) and the kernel launches it made */
int qpc_arnoldi_last_run(qpc_arnoldi* h, float* ms, int64_t* launches);

/* ---------------------------------------------------------------- surrogate network
 * No counterpart in the reference.  An ensemble of n_members MLPs, each
 * n_in -> n_layers x n_hidden (GELU) -> n_out, trained on the GPU with Adam:
 * bfloat16 operands, fp32 accumulation on the tensor cores, fp32 master weights,
 * biases, activations before rounding, loss gradient and optimiser state.  Loss:
 * mean squared error over rows and outputs.  Rows are float32 [n][n_in], targets
 * float32 [n][n_out]; n_hidden must be a multiple of 16 and n_out of 8. */
typedef struct qpc_mlp qpc_mlp;
int qpc_mlp_create(int32_t n_in, int32_t n_hidden, int32_t n_layers, int32_t n_out, int32_t n_members, uint64_t seed,
	qpc_mlp** out);
int qpc_mlp_destroy(qpc_mlp* h);
/* parameters per member; flat fp32 order W_0 [n_hidden][K0] (K0 = n_in rounded up to 16,
 * columns >= n_in unused), b_0, W_1, b_1, ..., W_last [n_out][n_hidden], b_last */
int qpc_mlp_param_count(qpc_mlp* h, int64_t* n);
int qpc_mlp_get_params(qpc_mlp* h, int32_t member, float* params);
int qpc_mlp_set_params(qpc_mlp* h, int32_t member, const float* params);
/* loss[member] and, if grad != NULL, grad[member][param_count] on the same n rows; no update */
int qpc_mlp_loss_grad(qpc_mlp* h, const float* X, const float* Y, int32_t n, float* loss, float* grad);
/* epochs of Adam (lr, beta 0.9 / 0.999, eps 1e-8) over minibatches of `batch` rows, each
 * member on its own shuffle drawn from seed; loss_hist [epochs][members] or NULL */
int qpc_mlp_train(qpc_mlp* h, const float* X, const float* Y, int32_t n, int32_t epochs, int32_t batch, float lr, uint64_t seed,
	float* loss_hist);
/* out [members][n][n_out] */
int qpc_mlp_predict(qpc_mlp* h, const float* X, int32_t n, float* out);

/* ---------------------------------------------------------------- no device allocation
 * No counterpart in the reference (it has no device code).  For callers that
 * cannot call cudaMalloc -- a framework that owns every device allocation
 * through its own pool, code running while a stream is being captured, or an
 * embedding with a fixed device-memory budget -- this entry point performs the
 * field-free Crank-Nicolson step of qpc_lgwz_propagate_free on buffers the
 * caller owns, and allocates nothing: its scratch is a fixed array
 * of 2 * QPC_NOALLOC_MAX_ELEMS complex128 values (32 MiB) compiled into the
 * library, which every GPU that loads the library holds until the process exits.
 *   coef  device, [n_inst][n_m][n_l][n_r] complex128, in/out
 *   S     device, [n_r][p+1] overlap band
 *   ffac  device, [lmax+1][n_r][p+1] complex128 with lmax = n_l - 1 + max(|m0|, |m0+n_m-1|)
 *         (channel (m, il) uses row l = il + |m|): the LDL^T factors of S + i dt/2 H_l,
 *         entries 0..p-1 of row r = L(r, r-1-c) and entry p = 1/D(r)
 *         (what qpc_ldlt_csym returns, packed per l)
 *   stream  a cudaStream_t (NULL = legacy default stream); the call only enqueues work
 * Limit: n_inst*n_m*n_l*n_r + ceil(n_inst/2) <= QPC_NOALLOC_MAX_ELEMS, otherwise
 * QPC_ERR_ARGS with a message.  The first call on a device looks up the
 * scratch's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.  The address is kept per
 * device for the CUDA runtime's primary context of that device (the context
 * cudaSetDevice makes current); a caller that makes its own driver-API context
 * current must not use this entry point.  All calls on a device share
 * the one scratch array and it keeps the previous call's contents, so calls
 * that overlap on the GPU (different streams or host threads) race: serialise
 * them.  Nothing in the scratch needs to start at zero: every call writes what
 * it later reads. */
#define QPC_NOALLOC_MAX_ELEMS (1L << 20)
int qpc_fieldfree_noalloc(const qpc_dims* dims, const double* S, const double* ffac, double* coef, void* stream);

/* ---------------------------------------------------------------- momentum spectra
 * Photoelectron momentum distributions of spherical/spectrum/momentum_1e.hpp: the
 * projection of the final state onto Coulomb (or plane) partial waves of
 * spectrum_c_pcs (443-514, measure_* 337-403), and the t-SURFF flux integral of
 * spectrum_c_tsf (516-1072), accumulated after every step (binsrc/sphTDSE.cpp:800,
 * 804, 940, 944).  Tables are built on the host; the contractions run on the GPU.
 * Angles: kt = polar angle theta_k, kp = azimuth phi_k. */
typedef struct qpc_kgrid {
	int32_t nkr, nkt, nkp;   /* points in |k|, theta_k, phi_k (spec_nkr/nkt/nkp) */
	double krmin, krmax;     /* |k| range; must give |k| > 0 everywhere */
	double ktmin, ktmax;     /* theta_k range (uniform, set_sequence_lin) */
	double kpmin, kpmax;     /* phi_k range (uniform) */
	int32_t flag;            /* 0: |k| uniform; 1: k^2/2 uniform (set_sequence_sqr), spectrum/inventory.h:15-39 */
} qpc_kgrid;

/* Building blocks of the tables (functions/coulomb.h, functions/basis_legendre.h):
 * F[l] = F_l(eta, rho), Fp[l] = dF_l/drho for l = 0..lmax, rho > 0 (Abramowitz-Stegun
 * normalisation); sigma[l] = arg Gamma(l + 1 + i eta); out[l(l+1)/2 + m] = Y_lm(theta, 0)
 * at x = cos(theta) with the Condon-Shortley phase, 0 <= m <= l <= lmax. */
int qpc_coulomb_f(double eta, double rho, int32_t lmax, double* F, double* Fp);
int qpc_coulomb_sigma(double eta, int32_t lmax, double* sigma);
int qpc_sph_legendre(int32_t lmax, double x, double* out);

/* spectrum_c_pcs::initialize with the analytic Coulomb waves of charge zc
 * (momentum_1e.hpp:453-485; initialize_kr 119-148, initialize_th/ph 11-50): kr[nkr],
 * kt[nkt], kp[nkp]; ijl[kr][l][r] = int B_r F_l(-zc/k, k r) w(r) dr / k with
 * w = 1/(1 + e^{-5 (r - rb)}) for rb > 0 (plane waves with zc = 0) else 1;
 * plm[kt][im][il] = Y_lm(kt, 0); exm[kp][im] = e^{i m kp}; cps[kr][l] = e^{i (sigma_l - l pi/2)},
 * complex arrays as (re, im); l = 0..lmax, lmax = max|m| + n_l - 1. */
int qpc_pcs_tables(const qpc_dims* dims, const double* knots, const qpc_kgrid* grid, double zc, double rb,
	double* kr, double* kt, double* kp, double* ijl, double* plm, double* exm, double* cps);

/* spectrum_c_pcs::initialize with numerical partial waves (momentum_1e.hpp:487-512, initialize_kr
 * 150-188), the projection the reference's driver uses for screened potentials: for
 * V = -(zc + zs e^{-sigma r})/r (pot; QPC_POTENTIAL_HYDROGENIC gives zs = 0) and mass 1, the regular
 * solution u_l(kr) of the radial equation, normalised to cos(delta) F_l + sin(delta) G_l with the
 * Coulomb functions of charge zc, replaces F_l in ijl, and cps[kr][l] = e^{i (Delta_l - l pi/2)} with
 * Delta_l = delta_l + sigma_l.  Same layouts as qpc_pcs_tables. */
int qpc_pcs_tables_numeric(const qpc_dims* dims, const double* knots, const qpc_kgrid* grid, const qpc_potential* pot,
	double* kr, double* kt, double* kp, double* ijl, double* plm, double* exm, double* cps);

/* spectrum_c_tsf::initialize (momentum_1e.hpp:778-866) at the surface r0 with Coulomb
 * correction zc: axes as above; the nb <= p+1 splines non-zero at r0 (ib active index,
 * b0 value, br derivative); j0[kr][l] = F_l(-zc/k, k r0)/k, jr[kr][l] = F'_l(-zc/k, k r0);
 * y0[kt][im][il] = Y_lm(kt, 0); e0[kp][im] = e^{i m kp}; pmat[3][im][il] = <l m|cos|l+1 m>,
 * <l m|sin e^{-i phi}|l+1 m+1>, <l m|sin e^{-i phi}|l-1 m+1> (basisfunc.hpp:222-259). */
int qpc_tsurff_tables(const qpc_dims* dims, const double* knots, const qpc_kgrid* grid, double r0, double zc,
	double* kr, double* kt, double* kp, int32_t* nb, int32_t* ib, double* b0, double* br, double* j0, double* jr,
	double* y0, double* e0, double* pmat);

enum { QPC_SPEC_LMD = 0, QPC_SPEC_PMD = 1, QPC_SPEC_PAD = 2 };

/* PCS projector on the GPU: the tables of qpc_pcs_tables (or the caller's own, same layouts),
 * for wavefunctions of dims (dims->n_inst is ignored). */
typedef struct qpc_pcs qpc_pcs;
int qpc_pcs_create(const qpc_dims* dims, const qpc_kgrid* grid, const double* kr, const double* ijl, const double* plm,
	const double* exm, const double* cps, qpc_pcs** out);
int qpc_pcs_destroy(qpc_pcs* h);
/* measure_lmd (kind QPC_SPEC_LMD), measure_prj (PMD) or measure_pad (PAD) of
 * momentum_1e.hpp:337-403 for n_inst wavefunctions c[inst][m][l][r] (device memory when
 * on_device != 0, else host).  out (host, complex128): LMD [inst][kr][im][il] =
 * sqrt(2/pi) cps <ijl|c>; PMD [inst][kr][kt][kp] = sqrt(2/pi) sum plm exm cps <ijl|c>;
 * PAD [inst][kr][kt] = 2 sqrt(k) sum plm cps <ijl|c>. */
int qpc_pcs_measure(qpc_pcs* h, int32_t kind, const double* coef, int32_t on_device, int32_t n_inst, double* out);
/* the same on the resident state of a propagator handle (every instance) */
int qpc_lgwz_pcs(qpc_lgwz* prop, qpc_pcs* h, int32_t kind, double* out);

/* t-SURFF accumulator on the GPU for dims->n_inst wavefunctions: the tables of
 * qpc_tsurff_tables; the spectrum work[inst][kr][kt][kp] and the clock (time and the
 * displacements int A dt per instance) start at zero (clearwork). */
typedef struct qpc_tsurff qpc_tsurff;
int qpc_tsurff_create(const qpc_dims* dims, const qpc_kgrid* grid, const double* kr, const double* kt, const double* kp,
	int32_t nb, const int32_t* ib, const double* b0, const double* br, const double* j0, const double* jr, const double* y0,
	const double* e0, const double* pmat, qpc_tsurff** out);
int qpc_tsurff_destroy(qpc_tsurff* h);
int qpc_tsurff_clear(qpc_tsurff* h);
enum { QPC_TSURFF_FREE = 0, QPC_TSURFF_Z = 1, QPC_TSURFF_XY = 2 };
/* spectrum_c_tsf::accumulate (momentum_1e.hpp:627-777) for every instance after a step of
 * length dt: mode QPC_TSURFF_FREE (a unused), QPC_TSURFF_Z with a[inst][2] = (A_z(t_i), A_z(t_i+1)),
 * QPC_TSURFF_XY with a[inst][4] = (A_x(t_i), A_x(t_i+1), A_y(t_i), A_y(t_i+1)); a is host memory.
 * coef: the wavefunctions c[inst][m][l][r] after the step (device when on_device != 0). */
int qpc_tsurff_accumulate(qpc_tsurff* h, int32_t mode, const double* a, double dt, const double* coef, int32_t on_device);
/* the same on the resident state of a propagator handle */
int qpc_lgwz_tsurff(qpc_lgwz* prop, qpc_tsurff* h, int32_t mode, const double* a, double dt);
int qpc_vgwr_tsurff(qpc_vgwr* prop, qpc_tsurff* h, int32_t mode, const double* a, double dt);
/* work[inst][kr][kt][kp] complex128 (host); clock[inst][4] = (time, disx, disy, disz) when not NULL */
int qpc_tsurff_get(qpc_tsurff* h, double* work, double* clock);
/* device time (CUDA events around the kernels) of the last qpc_pcs_measure / accumulate call */
int qpc_pcs_last_run(qpc_pcs* h, float* ms);
int qpc_tsurff_last_run(qpc_tsurff* h, float* ms);

#ifdef __cplusplus
}
#endif
#endif
