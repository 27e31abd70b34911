// Stand-in for Intel MKL's <mkl.h>, used ONLY to compile the unmodified reference
// headers (QPC-TDSE include/) into the test oracle under oracle/_ref/.
//
// Test infrastructure, not product code.  The routines the reference's
// time-stepping path actually calls (cblas ?gemm, ?gemm_batch_strided,
// LAPACKE_zhbev/dsbgv/dpbtrf/dstev) are forwarded to the OpenBLAS build that
// ships inside scipy (its symbols carry a "scipy_" prefix).  The batched
// strided GEMMs are written here as a loop of single GEMMs, which is the MKL
// definition of cblas_?gemm_batch_strided.  Every other MKL entry point named by
// the reference (sparse BLAS, DSS, PARDISO, FEAST, VML) is only declared so the
// headers parse; calling one aborts.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <complex>

#ifndef MKL_Complex16
#define MKL_Complex16 std::complex<double>
#endif
#ifndef MKL_Complex8
#define MKL_Complex8 std::complex<float>
#endif
#define MKL_INT int
typedef int lapack_int;

[[noreturn]] static inline void qpc_shim_unsupported(const char* what)
{
	std::fprintf(stderr, "oracle shim: MKL routine %s is not available in this harness\n", what);
	std::abort();
}

// ---------------------------------------------------------------- CBLAS
enum CBLAS_LAYOUT { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
typedef enum CBLAS_LAYOUT CBLAS_ORDER;

extern "C" {
void scipy_cblas_dgemm(int, int, int, int, int, int, double, const double*, int, const double*, int, double, double*, int);
void scipy_cblas_zgemm(int, int, int, int, int, int, const void*, const void*, int, const void*, int, const void*, void*, int);
void scipy_cblas_zdotc_sub(int, const void*, int, const void*, int, void*);
void scipy_cblas_daxpy(int, double, const double*, int, double*, int);
void scipy_cblas_zaxpy(int, const void*, const void*, int, void*, int);
int scipy_LAPACKE_zhbev(int, char, char, int, int, void*, int, double*, void*, int);
int scipy_LAPACKE_dsbgv(int, char, char, int, int, int, double*, int, double*, int, double*, double*, int);
int scipy_LAPACKE_dpbtrf(int, char, int, int, double*, int);
int scipy_LAPACKE_dstev(int, char, int, double*, double*, double*, int);
int scipy_LAPACKE_dsbev(int, char, char, int, int, double*, int, double*, double*, int);
}

static inline void cblas_dgemm(CBLAS_LAYOUT l, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, MKL_INT m, MKL_INT n, MKL_INT k,
	double alpha, const double* a, MKL_INT lda, const double* b, MKL_INT ldb, double beta, double* c, MKL_INT ldc)
{
	scipy_cblas_dgemm(l, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
static inline void cblas_zgemm(CBLAS_LAYOUT l, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, MKL_INT m, MKL_INT n, MKL_INT k,
	const void* alpha, const void* a, MKL_INT lda, const void* b, MKL_INT ldb, const void* beta, void* c, MKL_INT ldc)
{
	scipy_cblas_zgemm(l, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
static inline void cblas_dgemm_batch_strided(CBLAS_LAYOUT l, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb,
	MKL_INT m, MKL_INT n, MKL_INT k, double alpha, const double* a, MKL_INT lda, MKL_INT sa,
	const double* b, MKL_INT ldb, MKL_INT sb, double beta, double* c, MKL_INT ldc, MKL_INT sc, MKL_INT nb)
{
	for (MKL_INT i = 0; i < nb; ++i)
		scipy_cblas_dgemm(l, ta, tb, m, n, k, alpha, a + (long)i * sa, lda, b + (long)i * sb, ldb, beta, c + (long)i * sc, ldc);
}
static inline void cblas_zgemm_batch_strided(CBLAS_LAYOUT l, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb,
	MKL_INT m, MKL_INT n, MKL_INT k, const void* alpha, const void* a, MKL_INT lda, MKL_INT sa,
	const void* b, MKL_INT ldb, MKL_INT sb, const void* beta, void* c, MKL_INT ldc, MKL_INT sc, MKL_INT nb)
{
	const double* A = (const double*)a; const double* B = (const double*)b; double* C = (double*)c;
	for (MKL_INT i = 0; i < nb; ++i)
		scipy_cblas_zgemm(l, ta, tb, m, n, k, alpha, A + 2l * i * sa, lda, B + 2l * i * sb, ldb, beta, C + 2l * i * sc, ldc);
}
static inline void cblas_zdotc_sub(MKL_INT n, const void* x, MKL_INT ix, const void* y, MKL_INT iy, void* r) { scipy_cblas_zdotc_sub(n, x, ix, y, iy, r); }
static inline void cblas_daxpy(MKL_INT n, double a, const double* x, MKL_INT ix, double* y, MKL_INT iy) { scipy_cblas_daxpy(n, a, x, ix, y, iy); }
static inline void cblas_zaxpy(MKL_INT n, const void* a, const void* x, MKL_INT ix, void* y, MKL_INT iy) { scipy_cblas_zaxpy(n, a, x, ix, y, iy); }

// ---------------------------------------------------------------- LAPACKE
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
static inline lapack_int LAPACKE_zhbev(int lay, char jobz, char uplo, lapack_int n, lapack_int kd, MKL_Complex16* ab, lapack_int ldab, double* w, MKL_Complex16* z, lapack_int ldz)
{ return scipy_LAPACKE_zhbev(lay, jobz, uplo, n, kd, (void*)ab, ldab, w, (void*)z, ldz); }
static inline lapack_int LAPACKE_dsbgv(int lay, char jobz, char uplo, lapack_int n, lapack_int ka, lapack_int kb, double* ab, lapack_int ldab, double* bb, lapack_int ldbb, double* w, double* z, lapack_int ldz)
{ return scipy_LAPACKE_dsbgv(lay, jobz, uplo, n, ka, kb, ab, ldab, bb, ldbb, w, z, ldz); }
static inline lapack_int LAPACKE_dpbtrf(int lay, char uplo, lapack_int n, lapack_int kd, double* ab, lapack_int ldab)
{ return scipy_LAPACKE_dpbtrf(lay, uplo, n, kd, ab, ldab); }
static inline lapack_int LAPACKE_dstev(int lay, char jobz, lapack_int n, double* d, double* e, double* z, lapack_int ldz)
{ return scipy_LAPACKE_dstev(lay, jobz, n, d, e, z, ldz); }
static inline lapack_int LAPACKE_dsbev(int lay, char jobz, char uplo, lapack_int n, lapack_int kd, double* ab, lapack_int ldab, double* w, double* z, lapack_int ldz)
{ return scipy_LAPACKE_dsbev(lay, jobz, uplo, n, kd, ab, ldab, w, z, ldz); }

#define QPC_SHIM_UNSUPPORTED(ret, name) template <class... A> static inline ret name(A...) { qpc_shim_unsupported(#name); }
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_dgbsv)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_dgesv)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_dpbtrs)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_dposv)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_dppsv)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_dpttrf)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_dspev)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_dspgv)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_dsyev)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_dsyevd)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_zgbsv)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_zgesv)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_zpbtrf)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_zpbtrs)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_zposv)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_zppsv)
QPC_SHIM_UNSUPPORTED(lapack_int, LAPACKE_zpttrf)

// ---------------------------------------------------------------- VML (declared only)
#define QPC_SHIM_VML(name) template <class... A> static inline void name(A...) { qpc_shim_unsupported(#name); }
QPC_SHIM_VML(vdPow) QPC_SHIM_VML(vdAtan2) QPC_SHIM_VML(vdPowx) QPC_SHIM_VML(vdSqrt) QPC_SHIM_VML(vdCbrt)
QPC_SHIM_VML(vdInvSqrt) QPC_SHIM_VML(vdInvCbrt) QPC_SHIM_VML(vdPow3o2) QPC_SHIM_VML(vdPow2o3) QPC_SHIM_VML(vdExp)
QPC_SHIM_VML(vdLn) QPC_SHIM_VML(vdLog10) QPC_SHIM_VML(vdCos) QPC_SHIM_VML(vdSin) QPC_SHIM_VML(vdTan) QPC_SHIM_VML(vdAcos)
QPC_SHIM_VML(vdAsin) QPC_SHIM_VML(vdAtan) QPC_SHIM_VML(vdCosh) QPC_SHIM_VML(vdSinh) QPC_SHIM_VML(vdTanh) QPC_SHIM_VML(vdAcosh)
QPC_SHIM_VML(vdAsinh) QPC_SHIM_VML(vdAtanh)
QPC_SHIM_VML(vzSqrt) QPC_SHIM_VML(vzTanh) QPC_SHIM_VML(vzTan) QPC_SHIM_VML(vzSinh) QPC_SHIM_VML(vzSin) QPC_SHIM_VML(vzPow)
QPC_SHIM_VML(vzLog10) QPC_SHIM_VML(vzLn) QPC_SHIM_VML(vzCosh) QPC_SHIM_VML(vzCos) QPC_SHIM_VML(vzConj)
QPC_SHIM_VML(vzCIS) QPC_SHIM_VML(vzAtanh) QPC_SHIM_VML(vzAtan) QPC_SHIM_VML(vzAsinh) QPC_SHIM_VML(vzAsin) QPC_SHIM_VML(vzArg)
QPC_SHIM_VML(vzAcosh) QPC_SHIM_VML(vzAcos) QPC_SHIM_VML(vzAbs) QPC_SHIM_VML(vzMul) QPC_SHIM_VML(vzDiv)

// complex exponential of n values (the Arnoldi propagator's exp(-i dt a_k), la_1e.hpp:163-167)
static inline void vzExp(long long n, const MKL_Complex16* a, MKL_Complex16* y)
{
	const double* x = reinterpret_cast<const double*>(a);
	double* z = reinterpret_cast<double*>(y);
	for (long long i = 0; i < n; ++i) {
		std::complex<double> e = std::exp(std::complex<double>(x[2 * i], x[2 * i + 1]));
		z[2 * i] = e.real();
		z[2 * i + 1] = e.imag();
	}
}

static inline void mkl_set_num_threads(int) {}
static inline int mkl_get_max_threads() { return 1; }

// ---------------------------------------------------------------- sparse BLAS / checker (declared only)
typedef enum { SPARSE_STATUS_SUCCESS = 0, SPARSE_STATUS_NOT_INITIALIZED = 1, SPARSE_STATUS_ALLOC_FAILED = 2,
	SPARSE_STATUS_INVALID_VALUE = 3, SPARSE_STATUS_EXECUTION_FAILED = 4, SPARSE_STATUS_INTERNAL_ERROR = 5,
	SPARSE_STATUS_NOT_SUPPORTED = 6 } sparse_status_t;
typedef enum { SPARSE_OPERATION_NON_TRANSPOSE = 10, SPARSE_OPERATION_TRANSPOSE = 11, SPARSE_OPERATION_CONJUGATE_TRANSPOSE = 12 } sparse_operation_t;
typedef enum { SPARSE_MATRIX_TYPE_GENERAL = 20, SPARSE_MATRIX_TYPE_SYMMETRIC = 21, SPARSE_MATRIX_TYPE_HERMITIAN = 22,
	SPARSE_MATRIX_TYPE_TRIANGULAR = 23 } sparse_matrix_type_t;
typedef enum { SPARSE_INDEX_BASE_ZERO = 0, SPARSE_INDEX_BASE_ONE = 1 } sparse_index_base_t;
typedef enum { SPARSE_FILL_MODE_LOWER = 40, SPARSE_FILL_MODE_UPPER = 41, SPARSE_FILL_MODE_FULL = 42 } sparse_fill_mode_t;
typedef enum { SPARSE_DIAG_NON_UNIT = 50, SPARSE_DIAG_UNIT = 51 } sparse_diag_type_t;
struct sparse_matrix;
typedef struct sparse_matrix* sparse_matrix_t;
struct matrix_descr { sparse_matrix_type_t type; sparse_fill_mode_t mode; sparse_diag_type_t diag; };
typedef enum { MKL_ZERO_BASED = 0, MKL_ONE_BASED = 1 } sparse_matrix_indexing;
typedef enum { MKL_C_STYLE = 0, MKL_FORTRAN_STYLE = 1 } sparse_matrix_print_styles;
typedef enum { MKL_CSR = 0 } sparse_matrix_formats;
typedef enum { MKL_GENERAL_STRUCTURE = 0, MKL_UPPER_TRIANGULAR = 1, MKL_LOWER_TRIANGULAR = 2, MKL_STRUCTURAL_SYMMETRIC = 3 } sparse_matrix_structures;
typedef enum { MKL_NO_PRINT = 0, MKL_PRINT = 1 } sparse_matrix_message_levels;
typedef enum { MKL_SPARSE_CHECKER_SUCCESS = 0 } sparse_checker_error_values;
typedef struct sparse_struct {
	MKL_INT n, *csr_ia, *csr_ja, check_result[3];
	sparse_matrix_indexing indexing; sparse_matrix_structures matrix_structure;
	sparse_matrix_formats matrix_format; sparse_matrix_message_levels message_level;
	sparse_matrix_print_styles print_style;
} sparse_struct;
QPC_SHIM_UNSUPPORTED(void, sparse_matrix_checker_init)
QPC_SHIM_UNSUPPORTED(sparse_checker_error_values, sparse_matrix_checker)
QPC_SHIM_UNSUPPORTED(sparse_status_t, mkl_sparse_destroy)
QPC_SHIM_UNSUPPORTED(sparse_status_t, mkl_sparse_convert_csr)
QPC_SHIM_UNSUPPORTED(sparse_status_t, mkl_sparse_d_export_csr)
QPC_SHIM_UNSUPPORTED(sparse_status_t, mkl_sparse_z_export_csr)
QPC_SHIM_UNSUPPORTED(sparse_status_t, mkl_sparse_d_create_csr)
QPC_SHIM_UNSUPPORTED(sparse_status_t, mkl_sparse_z_create_csr)
QPC_SHIM_UNSUPPORTED(sparse_status_t, mkl_sparse_d_mv)
QPC_SHIM_UNSUPPORTED(sparse_status_t, mkl_sparse_z_mv)
QPC_SHIM_UNSUPPORTED(sparse_status_t, mkl_sparse_spmm)
QPC_SHIM_UNSUPPORTED(sparse_status_t, mkl_sparse_d_add)
QPC_SHIM_UNSUPPORTED(sparse_status_t, mkl_sparse_z_add)
QPC_SHIM_UNSUPPORTED(sparse_status_t, mkl_sparse_order)
QPC_SHIM_UNSUPPORTED(sparse_status_t, mkl_sparse_copy)

// ---------------------------------------------------------------- DSS / PARDISO / FEAST (declared only)
typedef void* _MKL_DSS_HANDLE_t;
#define MKL_DSS_SUCCESS 0
#define MKL_DSS_DEFAULTS 0
#define MKL_DSS_SYMMETRIC 536870976
#define MKL_DSS_SYMMETRIC_STRUCTURE 536871040
#define MKL_DSS_NON_SYMMETRIC 536871104
#define MKL_DSS_SYMMETRIC_COMPLEX 536871168
#define MKL_DSS_SYMMETRIC_STRUCTURE_COMPLEX 536871232
#define MKL_DSS_NON_SYMMETRIC_COMPLEX 536871296
#define MKL_DSS_POSITIVE_DEFINITE 134217792
#define MKL_DSS_INDEFINITE 134217856
#define MKL_DSS_HERMITIAN_POSITIVE_DEFINITE 134217920
#define MKL_DSS_HERMITIAN_INDEFINITE 134217984
QPC_SHIM_UNSUPPORTED(int, dss_create)
QPC_SHIM_UNSUPPORTED(int, dss_define_structure)
QPC_SHIM_UNSUPPORTED(int, dss_reorder)
QPC_SHIM_UNSUPPORTED(int, dss_factor_real)
QPC_SHIM_UNSUPPORTED(int, dss_factor_complex)
QPC_SHIM_UNSUPPORTED(int, dss_solve_real)
QPC_SHIM_UNSUPPORTED(int, dss_solve_complex)
QPC_SHIM_UNSUPPORTED(int, dss_delete)
QPC_SHIM_UNSUPPORTED(void, PARDISO)
QPC_SHIM_UNSUPPORTED(void, pardisoinit)
QPC_SHIM_UNSUPPORTED(void, feastinit)
QPC_SHIM_UNSUPPORTED(void, dfeast_scsrev)
QPC_SHIM_UNSUPPORTED(void, dfeast_scsrgv)
QPC_SHIM_UNSUPPORTED(void, zfeast_hcsrev)
QPC_SHIM_UNSUPPORTED(void, zfeast_hcsrgv)
